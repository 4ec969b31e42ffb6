// Design-matrix (A-matrix) assembly kernels.
//
// Reference: Cheby::Deriv_2B / Deriv_3B / Deriv_4B (src/Cheby.C:709-1729) with
// set_polys / set_polys_out_of_range (src/Cheby.C:207-443) and FCUT::get_fcut
// (src/Fcut.C:17-72).  The reference loops, per cluster, over every allowed power
// tuple p and scatters ~50-130 flops into the A rows of the cluster's atoms.
//
// GB300 formulation (same sums, different association):
//  * Force rows are gathered by their owner atom (one CTA per real atom), so
//    every A entry is written once, without atomics, in a fixed order.
//  * For an owner at canonical position pi of a cluster, the slots split into the
//    ones incident to it (I) and the rest (O).  The per-power derivative sum
//        F_x[p] = sum_{s in I} w_s,x h_s[p_s] prod_{s' != s} g_s'[p_s']
//    factorises as M_x[p_I] * Q[p_O]; M and Q are tabulated once per cluster in
//    shared memory, so each (cluster, power) costs 3 FMAs instead of ~40.
//  * Stress / energy rows are gathered per (frame, cluster type) with the split
//    S1 = I(0), S2 = O(0):  W_ab[p] = A1_ab[p1] Q2[p2] + Q1[p1] A2_ab[p2],
//    E[p] = Q1[p1] Q2[p2].
//  * Powers that PARAM_INDICES maps to one column (permutations of identical
//    atoms) are contiguous; they are summed in shared memory before the store.
// g_s[n] = fcut_s T_n(x_s), h_s[n] = d g_s[n] / dr_s.
#include <algorithm>
#include <cstdio>
#include "assemble.h"
#include "basis.cuh"

namespace cgd {

// ---------------------------------------------------------------- slot tables
// Canonical slot lists: incident slots of canonical position pi, and the rest.
__device__ __forceinline__ void role_slots(int NB, int pi, int* I, int* O) {
    for (int k = 0; k < NB - 1; ++k) I[k] = role_slot_in(NB, pi, k);
    for (int k = 0; k < (NB == 3 ? 1 : 3); ++k) O[k] = role_slot_out(NB, pi, k);
}

// Basis of the edge that maps to canonical slot s of cluster q: g, h (ord values each,
// in the compute type T), the edge's vector oriented first->second actual member, and
// its length.  The distance and cut-off are FP64 in both forms.
struct SlotBasis {
    int e, ma, mb;
    double r, rab[3];
};

// The edge of cluster id that maps to canonical slot s, and its two members.
__device__ __forceinline__ int slot_edge(const ModelDev& M, int NB, int id, int s, int& a, int& b) {
    const int np = NB == 3 ? 3 : 6;
    const int8_t* pm = (NB == 3 ? M.pidx3 : M.pidx4) + id * np;
    int e = 0;
    for (int k = 0; k < np; ++k) if (pm[k] == s) e = k;
    edge_members(NB, e, a, b);
    return e;
}

template <typename TC>
__device__ void slot_basis(const ModelDev& M, const FramesDev& F, int NB, int f, int4 mem, int id, int T,
                           int s, int ord, TC* g, TC* h, SlotBasis& sb) {
    int a, b;
    const int e = slot_edge(M, NB, id, s, a, b);
    const int N = F.natoms[f];
    const int64_t gb = F.ghost_ofs[f];
    const int ga = member(mem, a), gbm = member(mem, b);
    const BoxDev& B = F.box[f];
    sb.e = e; sb.ma = a; sb.mb = b;
    sb.r = dist_exact(B.h, F.scaled + 3 * (gb + ga), F.scaled + 3 * (gb + gbm), sb.rab);
    const ClusterTypeDev& CT = (NB == 3 ? M.types3 : M.types4)[T];
    const int* typ = F.type + F.atom_ofs[f];
    const int pt = M.int_pair_map[typ[ga % N] * M.natmtyp + typ[gbm % N]];
    double fc, fd;
    fcut_eval(M, sb.r, CT.smax[s], fc, fd);
    basis_gh_t<TC>(M, M.pairs[pt].lambda, CT.xavg[s], CT.xdiff[s], CT.smin[s], sb.r, 0, ord, fc, fd, g, h, 1);
}

// ---------------------------------------------------------------- per-cluster slot bases
// One thread per (cluster, slot) of the batch: g, h, r and r_ab of the slot's edge,
// [cluster][slot][2 ord + 4].  The force kernel visits every cluster once per member
// atom and the stress/energy kernel once more; with these tables the basis is
// evaluated once per cluster.
template <int NBODY, typename R>
__global__ void k_cluster_basis(ModelDev M, FramesDev F, ClusterSet CS, int64_t nq, R* __restrict__ out) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    const int ord = NBODY == 3 ? M.order3 : M.order4;
    const int stride = 2 * ord + 4;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nq * NP; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t q = t / NP;
        const int s = (int)(t % NP);
        int lo = 0, hi = F.nframes - 1;   // frame of cluster q: last f with its first cluster <= q
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (CS.ofs[F.atom_ofs[mid]] <= q) lo = mid; else hi = mid - 1;
        }
        const int f = lo;
        const int N = F.natoms[f];
        const int* typ = F.type + F.atom_ofs[f];
        const int4 mm = CS.m[q];
        int id = 0, w = 1;
        for (int u = 0; u < NBODY; ++u) { id += w * (typ[member(mm, u) % N] + 1); w *= 10; }
        R* o = out + t * stride;
        SlotBasis sb;
        slot_basis<R>(M, F, NBODY, f, mm, id, CS.type[q], s, ord, o, o + ord, sb);
        o[2 * ord] = R(sb.r);
        o[2 * ord + 1] = R(sb.rab[0]); o[2 * ord + 2] = R(sb.rab[1]); o[2 * ord + 3] = R(sb.rab[2]);
    }
}

// ---------------------------------------------------------------- 2-body force rows
// One CTA per real atom; threads over the 2-body columns (pair type, n).
template <typename R>
__global__ void k_force2(ModelDev M, FramesDev F, NeighDev NB, Buckets inc, const int64_t* key_frame_ofs, R* A,
                         int64_t lda) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ord = M.order2;
    const int ncol = M.npairs * ord;
    R* sD = reinterpret_cast<R*>(smem_raw);            // [chunk][3*ord]
    int* sPt = reinterpret_cast<int*>(sD + (size_t)blockDim.x * 3 * ord);
    const int gatom = blockIdx.x;
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (F.atom_ofs[mid] <= gatom) lo = mid; else hi = mid - 1; }
    const int f = lo;
    const int a = gatom - (int)F.atom_ofs[f];
    const BoxDev& B = F.box[f];
    const int64_t kb = key_frame_ofs[f];
    const int64_t e0 = inc.key_ofs[kb + a], e1 = inc.key_ofs[kb + a + 1];
    const int64_t pbase = NB.ofs2[F.atom_ofs[f]];   // first 2B pair of the frame
    constexpr int MAXC = 8;
    R acc[MAXC][3];
    for (int c = 0; c < MAXC; ++c) acc[c][0] = acc[c][1] = acc[c][2] = R(0);
    for (int64_t c0 = e0; c0 < e1; c0 += blockDim.x) {
        const int64_t ei = c0 + threadIdx.x;
        if (ei < e1) {
            const int v = inc.val[ei];
            const int64_t p = pbase + (v >> 1);
            const double sgn = (v & 1) ? -1.0 : 1.0;
            const int pt = NB.pt2[p];
            const double r = NB.r2[p];
            const PairDev P = M.pairs[pt];
            double fc, fd;
            fcut_eval(M, r, P.smax, fc, fd);
            const double ir = sgn * B.perm2 / r;
            const R ux = R(NB.rab2[3 * p] * ir), uy = R(NB.rab2[3 * p + 1] * ir), uz = R(NB.rab2[3 * p + 2] * ir);
            R* d = sD + (size_t)threadIdx.x * 3 * ord;
            // h_n (n = 1..ord) into the x slot, then spread to y and z (recursion in R)
            basis_gh_t<R>(M, P.lambda, P.xavg, P.xdiff, P.smin, r, 1, ord, fc, fd, d + 1, d, 3);
            for (int n = 0; n < ord; ++n) {
                const R t = d[3 * n];
                d[3 * n] = t * ux; d[3 * n + 1] = t * uy; d[3 * n + 2] = t * uz;
            }
            sPt[threadIdx.x] = pt;
        }
        __syncthreads();
        const int cnt = (int)min((int64_t)blockDim.x, e1 - c0);
        for (int c = 0; c < MAXC; ++c) {
            const int col = threadIdx.x + c * blockDim.x;
            if (col >= ncol) break;
            const int pt = col / ord, n = col % ord;
            for (int k = 0; k < cnt; ++k) {
                if (sPt[k] != pt) continue;
                const R* d = sD + (size_t)k * 3 * ord + 3 * n;
                acc[c][0] += d[0]; acc[c][1] += d[1]; acc[c][2] += d[2];
            }
        }
        __syncthreads();
    }
    const int64_t row = F.row_ofs[f] + 3 * a;
    for (int c = 0; c < MAXC; ++c) {
        const int col = threadIdx.x + c * blockDim.x;
        if (col >= ncol) break;
        const int base = M.pairs[col / ord].col;   // HIERARC: excluded pairs have no columns
        if (base < 0) continue;
        const int oc = base + col % ord;
        A[(row + 0) * lda + oc] = acc[c][0];
        A[(row + 1) * lda + oc] = acc[c][1];
        A[(row + 2) * lda + oc] = acc[c][2];
    }
}

// ---------------------------------------------------------------- 2-body stress/energy rows
// grid: (frame, slice of the frame's pairs); threads over the 2-body columns.  Each
// CTA sums its slice into per-column partials (comps: 0 E, 1 xx, 2 yy, 3 zz, 4 xy,
// 5 xz, 6 yz); k_virial2_rows adds a frame's slices in slice order and writes the
// rows, so the result does not depend on timing.  The slices spread a block's few
// frames over every SM (the pairs' FP64 basis evaluations dominate this kernel).
template <typename R, int MAXC>
__global__ void k_virial2(ModelDev M, FramesDev F, NeighDev NB, int nslice, R* __restrict__ part) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ord = M.order2;
    const int ncol = M.npairs * ord;
    const int f = blockIdx.x, sl = blockIdx.y;
    const int srows = F.stress_rows[f], erows = F.energy_rows[f];
    if (srows == 0 && erows == 0) return;
    R* sGH = reinterpret_cast<R*>(smem_raw);                      // [chunk][2*ord]
    R* sV = sGH + (size_t)blockDim.x * 2 * ord;                    // [chunk][6]
    int* sPt = reinterpret_cast<int*>(sV + (size_t)blockDim.x * 6);
    const BoxDev& B = F.box[f];
    const int64_t q0 = NB.ofs2[F.atom_ofs[f]], q1 = NB.ofs2[F.atom_ofs[f + 1]];
    const int64_t len = (q1 - q0 + nslice - 1) / nslice;
    const int64_t p0 = min(q1, q0 + (int64_t)sl * len), p1 = min(q1, p0 + len);
    R acc[MAXC][7];   // MAXC columns per thread, unrolled so that acc stays in registers
    for (int c = 0; c < MAXC; ++c) for (int k = 0; k < 7; ++k) acc[c][k] = R(0);
    for (int64_t c0 = p0; c0 < p1; c0 += blockDim.x) {
        const int64_t p = c0 + threadIdx.x;
        if (p < p1) {
            const int pt = NB.pt2[p];
            const double r = NB.r2[p];
            const PairDev P = M.pairs[pt];
            double fc, fd;
            fcut_eval(M, r, P.smax, fc, fd);
            R* gh = sGH + (size_t)threadIdx.x * 2 * ord;
            basis_gh_t<R>(M, P.lambda, P.xavg, P.xdiff, P.smin, r, 1, ord, B.perm2 * fc, B.perm2 * fd, gh, gh + 1, 2);
            const double* x = NB.rab2 + 3 * p;
            R* v = sV + (size_t)threadIdx.x * 6;
            if constexpr (sizeof(R) == 8) {
                v[0] = x[0] * x[0] / r; v[1] = x[1] * x[1] / r; v[2] = x[2] * x[2] / r;
                v[3] = x[0] * x[1] / r; v[4] = x[0] * x[2] / r; v[5] = x[1] * x[2] / r;
            } else {   // r_a r_b / r in FP32
                const R xf[3] = {R(x[0]), R(x[1]), R(x[2])}, rf = R(r);
                v[0] = xf[0] * xf[0] / rf; v[1] = xf[1] * xf[1] / rf; v[2] = xf[2] * xf[2] / rf;
                v[3] = xf[0] * xf[1] / rf; v[4] = xf[0] * xf[2] / rf; v[5] = xf[1] * xf[2] / rf;
            }
            sPt[threadIdx.x] = pt;
        }
        __syncthreads();
        const int cnt = (int)min((int64_t)blockDim.x, p1 - c0);
#pragma unroll
        for (int c = 0; c < MAXC; ++c) {
            const int col = threadIdx.x + c * blockDim.x;
            if (col < ncol) {
                const int pt = col / ord, n = col % ord;
                for (int k = 0; k < cnt; ++k) {
                    if (sPt[k] != pt) continue;
                    const R* gh = sGH + (size_t)k * 2 * ord + 2 * n;
                    const R* v = sV + (size_t)k * 6;
                    acc[c][0] += gh[0];
#pragma unroll
                    for (int q = 0; q < 6; ++q) acc[c][1 + q] -= gh[1] * v[q];
                }
            }
        }
        __syncthreads();
    }
    R* o = part + ((int64_t)f * nslice + sl) * 7 * ncol;
#pragma unroll
    for (int c = 0; c < MAXC; ++c) {
        const int col = threadIdx.x + c * blockDim.x;
        if (col < ncol)
#pragma unroll
            for (int k = 0; k < 7; ++k) o[(int64_t)k * ncol + col] = acc[c][k];
    }
}

template <typename R>
__global__ void k_virial2_rows(ModelDev M, FramesDev F, int nslice, const R* __restrict__ part, R* A, int64_t lda) {
    const int ord = M.order2;
    const int ncol = M.npairs * ord;
    const int f = blockIdx.x;
    if (F.stress_rows[f] == 0 && F.energy_rows[f] == 0) return;
    const double inv_vol = 1.0 / F.box[f].vol;
    const R* o = part + (int64_t)f * nslice * 7 * ncol;
    for (int col = threadIdx.x; col < ncol; col += blockDim.x) {
        const int base = M.pairs[col / ord].col;   // HIERARC: excluded pairs have no columns
        if (base < 0) continue;
        R s[7];
        for (int k = 0; k < 7; ++k) s[k] = R(0);
        for (int sl = 0; sl < nslice; ++sl)
            for (int k = 0; k < 7; ++k) s[k] += o[((int64_t)sl * 7 + k) * ncol + col];
        write_virial_rows(F, f, base + col % ord, s, inv_vol, A, lda);
    }
}

// ---------------------------------------------------------------- owner incidence sort
// The owner's incidences inc.val[c0 .. c0 + nent) (cluster << 2 | member) sorted
// stably by key = cluster type * 4 + the owner's canonical role: sEnt[k] = entry k,
// sKey[k] its key, sOrd the entries in key order, and sCnt[key] the end of each key's
// run (its start is the previous key's end).  Every thread of the CTA calls it; the
// first barrier keeps a previous pass's readers of sCnt ahead of the reset.
template <int NBODY>
__device__ void sort_incidences(const ClusterSet& CS, const Buckets& inc, const int8_t* revs, const int* typ, int N,
                                int64_t qbase, int64_t c0, int nent, int nkeys, int* sEnt, int* sKey, int* sOrd,
                                int* sCnt) {
    const int lane = threadIdx.x & 31;
    __syncthreads();
    for (int k = threadIdx.x; k <= nkeys; k += blockDim.x) sCnt[k] = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < nent; k += blockDim.x) {
        const int v = inc.val[c0 + k];
        const int q = v >> 2, m = v & 3;
        const int4 mm = CS.m[qbase + q];
        const int T = CS.type[qbase + q];
        int id = 0, w = 1;
        for (int t = 0; t < NBODY; ++t) { id += w * (typ[member(mm, t) % N] + 1); w *= 10; }
        const int pi = revs[id * NBODY + m];
        sEnt[k] = v;
        sKey[k] = T * 4 + pi;
        atomicAdd(&sCnt[T * 4 + pi + 1], 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) for (int k = 1; k <= nkeys; ++k) sCnt[k] += sCnt[k - 1];
    __syncthreads();
    if (threadIdx.x < 32) {   // stable placement by (type, role), 32 entries at a time
        for (int b = 0; b < nent; b += 32) {
            const int k = b + lane;
            const bool act = k < nent;
            const int key = act ? sKey[k] : -1 - lane;
            const unsigned peers = __match_any_sync(0xffffffffu, key);
            const int leader = __ffs(peers) - 1;
            const int rank = __popc(peers & ((1u << lane) - 1u));
            int st = 0;
            if (act && lane == leader) st = sCnt[key];
            st = __shfl_sync(0xffffffffu, st, leader);
            if (act) sOrd[st + rank] = k;
            __syncwarp();
            if (act && lane == leader) sCnt[key] = st + __popc(peers);
            __syncwarp();
        }
    }
    __syncthreads();
}

// ---------------------------------------------------------------- many-body force rows
// One CTA per real (owner) atom.  PPT powers per thread cover every allowed power
// tuple of the largest cluster type, so the accumulators stay in registers.
// NT threads per CTA: MB_THREADS, or twice that for the 4-body kernel, whose one CTA
// per SM (shared-memory bound) then keeps 32 warps issuing instead of 16.
template <int NBODY, typename R, int PPT, int NT = MB_THREADS>
__global__ void __launch_bounds__(NT, NBODY == 3 ? (sizeof(R) == 4 ? 3 : 2) : 1) k_force_mb(ModelDev M, FramesDev F, ClusterSet CS, Buckets inc,
                                                         const int64_t* key_frame_ofs, const R* __restrict__ pre,
                                                         R* A, int64_t lda) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    constexpr int NI = NBODY - 1;
    constexpr int NO = NP - NI;
    constexpr int CB = mb_force_cb((int)sizeof(R));
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ord = NBODY == 3 ? M.order3 : M.order4;
    const int ntypes = NBODY == 3 ? M.ntypes3 : M.ntypes4;
    const ClusterTypeDev* types = NBODY == 3 ? M.types3 : M.types4;
    const uint8_t* pows = NBODY == 3 ? M.pow3 : M.pow4;
    const int* grps = NBODY == 3 ? M.grp3 : M.grp4;
    const int8_t* revs = NBODY == 3 ? M.rev3 : M.rev4;
    int sizeI = 1, sizeO = 1;
    for (int k = 0; k < NI; ++k) sizeI *= ord;
    for (int k = 0; k < NO; ++k) sizeO *= ord;
    const int per = 3 * sizeI + sizeO;
    const int nkeys = ntypes * 4;
    int max_allowed = 0;
    for (int t = 0; t < ntypes; ++t) max_allowed = max(max_allowed, types[t].n_allowed);
    const MbForceSmem L = mb_force_smem(NBODY, ord, nkeys, max_allowed, (int)sizeof(R));
    int* sEnt = reinterpret_cast<int*>(smem_raw + L.ent);
    int* sKey = reinterpret_cast<int*>(smem_raw + L.key);
    int* sOrd = reinterpret_cast<int*>(smem_raw + L.ord);
    int* sCnt = reinterpret_cast<int*>(smem_raw + L.cnt);
    int* sQ = reinterpret_cast<int*>(smem_raw + L.q);
    int* sPi = reinterpret_cast<int*>(smem_raw + L.pi);
    int* sSg = reinterpret_cast<int*>(smem_raw + L.sg);   // owner's sign on each slot's edge: +1, -1, 0
    R* sGH = reinterpret_cast<R*>(smem_raw + L.gh);
    R* sW = reinterpret_cast<R*>(smem_raw + L.w);
    R* sTab = reinterpret_cast<R*>(smem_raw + L.tab);

    const int gatom = blockIdx.x;
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (F.atom_ofs[mid] <= gatom) lo = mid; else hi = mid - 1; }
    const int f = lo;
    const int a = gatom - (int)F.atom_ofs[f];
    const int N = F.natoms[f];
    const BoxDev& B = F.box[f];
    const double perm = NBODY == 3 ? B.perm3 : B.perm4;
    const int64_t kb = key_frame_ofs[f];
    const int64_t e0 = inc.key_ofs[kb + a], e1 = inc.key_ofs[kb + a + 1];
    const bool single_pass = (e1 - e0) <= MB_MAX_ENT;
    const int64_t qbase = CS.ofs[F.atom_ofs[f]];
    const int* typ = F.type + F.atom_ofs[f];
    const int64_t row = F.row_ofs[f] + 3 * (int64_t)a;

    for (int64_t c0 = e0; c0 < e1; c0 += MB_MAX_ENT) {
        const int nent = (int)min((int64_t)MB_MAX_ENT, e1 - c0);
        sort_incidences<NBODY>(CS, inc, revs, typ, N, qbase, c0, nent, nkeys, sEnt, sKey, sOrd, sCnt);
        for (int T = 0; T < ntypes; ++T) {
            const int gbeg = T == 0 ? 0 : sCnt[T * 4 - 1], gend = sCnt[T * 4 + 3];
            if (gbeg == gend) continue;
            const ClusterTypeDev& CT = types[T];
            R acc[PPT][3];
#pragma unroll
            for (int k = 0; k < PPT; ++k) acc[k][0] = acc[k][1] = acc[k][2] = R(0);
            for (int pi = 0; pi < NBODY; ++pi) {
                const int key = T * 4 + pi;
                const int rb = key == 0 ? 0 : sCnt[key - 1], re = sCnt[key];
                if (rb == re) continue;
                int I[3], O[3];
                role_slots(NBODY, pi, I, O);
                int idxI[PPT], idxO[PPT];
#pragma unroll
                for (int k = 0; k < PPT; ++k) {
                    const int p = threadIdx.x + k * blockDim.x;
                    idxI[k] = -1; idxO[k] = 0;
                    if (p < CT.n_allowed) {
                        const uint8_t* pw = pows + CT.pow_offset + (size_t)p * NP;
                        int ii = 0, oo = 0;
                        for (int t = NI - 1; t >= 0; --t) ii = ii * ord + pw[I[t]];
                        for (int t = NO - 1; t >= 0; --t) oo = oo * ord + pw[O[t]];
                        idxI[k] = ii; idxO[k] = oo;
                    }
                }
                for (int b0 = rb; b0 < re; b0 += CB) {
                    const int nb = min(CB, re - b0);
                    if (threadIdx.x < nb) {
                        const int v = sEnt[sOrd[b0 + threadIdx.x]];
                        sQ[threadIdx.x] = v >> 2; sPi[threadIdx.x] = v & 3;
                        if (pre) {
                            const int4 mm = CS.m[qbase + (v >> 2)];
                            int id = 0, w = 1;
                            for (int u = 0; u < NBODY; ++u) { id += w * (typ[member(mm, u) % N] + 1); w *= 10; }
                            for (int s = 0; s < NP; ++s) {
                                int ea, eb;
                                slot_edge(M, NBODY, id, s, ea, eb);
                                sSg[threadIdx.x * NP + s] = ((v & 3) == ea) ? 1 : (((v & 3) == eb) ? -1 : 0);
                            }
                        }
                    }
                    __syncthreads();
                    // (1) per (cluster, slot): basis and the owner's weight vector
                    if (pre) {   // bases of the cluster tables, one thread per (cluster, slot, power)
                        const int stride = 2 * ord + 4;
                        for (int t = threadIdx.x; t < nb * NP * ord; t += blockDim.x) {
                            const int c = t / (NP * ord), rem = t % (NP * ord), s = rem / ord, n = rem % ord;
                            const R* src = pre + ((size_t)(qbase + sQ[c]) * NP + s) * stride;
                            const R ir = R(sSg[c * NP + s]) / src[2 * ord];   // sign / r in the form's type
                            const R wx = src[2 * ord + 1] * ir, wy = src[2 * ord + 2] * ir, wz = src[2 * ord + 3] * ir;
                            R* g = sGH + ((size_t)c * NP + s) * 2 * ord;
                            const R gn = src[n], hn = src[ord + n];
                            g[n] = gn; g[ord + n] = hn;
                            R* hw = sW + ((size_t)c * NP + s) * 3 * ord;
                            hw[n] = hn * wx; hw[ord + n] = hn * wy; hw[2 * ord + n] = hn * wz;
                        }
                    } else
                    for (int t = threadIdx.x; t < nb * NP; t += blockDim.x) {
                        const int c = t / NP, s = t % NP;
                        const int4 mm = CS.m[qbase + sQ[c]];
                        int id = 0, w = 1;
                        for (int u = 0; u < NBODY; ++u) { id += w * (typ[member(mm, u) % N] + 1); w *= 10; }
                        SlotBasis sb;
                        R* g = sGH + ((size_t)c * NP + s) * 2 * ord;
                        slot_basis<R>(M, F, NBODY, f, mm, id, T, s, ord, g, g + ord, sb);
                        const int m = sPi[c];
                        const double sg = (m == sb.ma) ? 1.0 : ((m == sb.mb) ? -1.0 : 0.0);
                        const double ir = sg / sb.r;
                        const R wx = R(sb.rab[0] * ir), wy = R(sb.rab[1] * ir), wz = R(sb.rab[2] * ir);
                        R* hw = sW + ((size_t)c * NP + s) * 3 * ord;   // h_s[n] * w_s,{x,y,z}
                        const R* h = g + ord;
                        for (int n = 0; n < ord; ++n) { hw[n] = h[n] * wx; hw[ord + n] = h[n] * wy; hw[2 * ord + n] = h[n] * wz; }
                    }
                    __syncthreads();
                    // (2) M_x,y,z over the incident-slot powers, Q over the others
                    const int nzt = sizeI + sizeO;   // M entries (x,y,z written together) + Q entries
                    for (int t = threadIdx.x; t < nb * nzt; t += blockDim.x) {
                        const int c = t / nzt, z = t % nzt;
                        const R* GH = sGH + (size_t)c * NP * 2 * ord;
                        const R* HW = sW + (size_t)c * NP * 3 * ord;
                        R* tab = sTab + (size_t)c * per;
                        if (z < sizeI) {
                            int pwr[3] = {0, 0, 0}, zz = z;
                            for (int u = 0; u < NI; ++u) { pwr[u] = zz % ord; zz /= ord; }
                            R gs[3];
                            for (int u = 0; u < NI; ++u) gs[u] = GH[(size_t)I[u] * 2 * ord + pwr[u]];
                            R other[3];   // product of the other incident slots' g
                            if (NI == 2) { other[0] = gs[1]; other[1] = gs[0]; }
                            else { other[0] = gs[1] * gs[2]; other[1] = gs[0] * gs[2]; other[2] = gs[0] * gs[1]; }
                            R mx = 0, my = 0, mz = 0;
                            for (int u = 0; u < NI; ++u) {
                                const R* hw = HW + (size_t)I[u] * 3 * ord + pwr[u];
                                mx += hw[0] * other[u]; my += hw[ord] * other[u]; mz += hw[2 * ord] * other[u];
                            }
                            tab[z] = mx; tab[sizeI + z] = my; tab[2 * sizeI + z] = mz;
                        } else {
                            int zz = z - sizeI;
                            R prod = R(1);
                            for (int u = 0; u < NO; ++u) { prod *= GH[(size_t)O[u] * 2 * ord + zz % ord]; zz /= ord; }
                            tab[3 * sizeI + (z - sizeI)] = prod;
                        }
                    }
                    __syncthreads();
                    // (3) 3 FMAs per (cluster, power)
                    for (int c = 0; c < nb; ++c) {
                        const R* tab = sTab + (size_t)c * per;
#pragma unroll
                        for (int k = 0; k < PPT; ++k) {
                            if (idxI[k] < 0) continue;
                            const R qv = tab[3 * sizeI + idxO[k]];
                            acc[k][0] += tab[idxI[k]] * qv;
                            acc[k][1] += tab[sizeI + idxI[k]] * qv;
                            acc[k][2] += tab[2 * sizeI + idxI[k]] * qv;
                        }
                    }
                    __syncthreads();
                }
            }
            // sum the powers that share a column, then store the owner's 3 rows
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
                const int p = threadIdx.x + k * blockDim.x;
                if (p < CT.n_allowed) {
                    sTab[3 * p] = acc[k][0]; sTab[3 * p + 1] = acc[k][1]; sTab[3 * p + 2] = acc[k][2];
                }
            }
            __syncthreads();
            const int* gp = grps + CT.grp_offset;
            for (int col = threadIdx.x; col < CT.n_true; col += blockDim.x) {
                R sx = 0, sy = 0, sz = 0;
                for (int p = gp[col]; p < gp[col + 1]; ++p) { sx += sTab[3 * p]; sy += sTab[3 * p + 1]; sz += sTab[3 * p + 2]; }
                const int64_t cc = CT.col_base + col;
                R* a0 = A + (row + 0) * lda + cc;
                R* a1 = A + (row + 1) * lda + cc;
                R* a2 = A + (row + 2) * lda + cc;
                if (single_pass) { *a0 = R(sx * perm); *a1 = R(sy * perm); *a2 = R(sz * perm); }
                else { *a0 += R(sx * perm); *a1 += R(sy * perm); *a2 += R(sz * perm); }
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------- many-body force rows, range form
// One CTA per owner atom, as k_force_mb, with the powers split differently: each
// thread takes a contiguous range of S = ceil(n_allowed / NT) powers of a cluster
// type.  The powers of one column are contiguous, so most columns fall to one thread
// and are summed in its FMA chain; a column whose powers cross a range boundary is
// finished by the thread holding its first power, which adds its neighbours' partial
// sums from shared memory in thread order (so the result does not depend on timing).
// The clusters of every owner role of a type are tabulated together, CB at a time,
// and each thread reads each power's table entries for each role from offsN.  With no
// per-power accumulator arrays two CTAs fit on an SM, and one CTA's table building
// and barriers overlap the other's FMAs.  blockDim.x (at most rg_max_threads) is chosen
// by the host (rg_threads).  The frame's PERM_SCALE is folded into the Q table.
template <int NBODY, typename R>
__global__ void __launch_bounds__(rg_max_threads((int)sizeof(R)), 2) k_force_rg(ModelDev M, FramesDev F, ClusterSet CS, Buckets inc,
                                                    const int64_t* key_frame_ofs, const R* __restrict__ pre,
                                                    R* A, int64_t lda) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    constexpr int NI = NBODY - 1;
    constexpr int NO = NP - NI;
    constexpr int CB = mb_force_cb((int)sizeof(R));
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ord = NBODY == 3 ? M.order3 : M.order4;
    const int ntypes = NBODY == 3 ? M.ntypes3 : M.ntypes4;
    const ClusterTypeDev* types = NBODY == 3 ? M.types3 : M.types4;
    const int* grps = NBODY == 3 ? M.grp3 : M.grp4;
    const int8_t* revs = NBODY == 3 ? M.rev3 : M.rev4;
    const uint4* offs = NBODY == 3 ? M.offs3 : M.offs4;
    const int* tcol = NBODY == 3 ? M.tcol3 : M.tcol4;
    int sizeI = 1, sizeO = 1;
    for (int k = 0; k < NI; ++k) sizeI *= ord;
    for (int k = 0; k < NO; ++k) sizeO *= ord;
    const int per = 3 * sizeI + sizeO;
    const int nkeys = ntypes * 4;
    const int NT = blockDim.x;
    const MbRangeSmem L = mb_range_smem(NBODY, ord, nkeys, NT, (int)sizeof(R));
    int* sEnt = reinterpret_cast<int*>(smem_raw + L.ent);
    int* sKey = reinterpret_cast<int*>(smem_raw + L.key);
    int* sOrd = reinterpret_cast<int*>(smem_raw + L.ord);
    int* sCnt = reinterpret_cast<int*>(smem_raw + L.cnt);
    int* sQ = reinterpret_cast<int*>(smem_raw + L.q);
    int* sM = reinterpret_cast<int*>(smem_raw + L.m);        // owner's member index in each cluster
    int* sRole = reinterpret_cast<int*>(smem_raw + L.role);  // owner's canonical role in each cluster
    int* sSg = reinterpret_cast<int*>(smem_raw + L.sg);      // owner's sign on each slot's edge: +1, -1, 0
    R* sGH = reinterpret_cast<R*>(smem_raw + L.gh);
    R* sW = reinterpret_cast<R*>(smem_raw + L.w);
    R* sTab = reinterpret_cast<R*>(smem_raw + L.tab);
    R* sPart = reinterpret_cast<R*>(smem_raw + L.part);

    const int gatom = blockIdx.x;
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) { int mid = (lo + hi + 1) >> 1; if (F.atom_ofs[mid] <= gatom) lo = mid; else hi = mid - 1; }
    const int f = lo;
    const int a = gatom - (int)F.atom_ofs[f];
    const int N = F.natoms[f];
    const BoxDev& B = F.box[f];
    const double perm = NBODY == 3 ? B.perm3 : B.perm4;
    const int64_t kb = key_frame_ofs[f];
    const int64_t e0 = inc.key_ofs[kb + a], e1 = inc.key_ofs[kb + a + 1];
    const bool single_pass = (e1 - e0) <= MB_MAX_ENT;
    const int64_t qbase = CS.ofs[F.atom_ofs[f]];
    const int* typ = F.type + F.atom_ofs[f];
    R* const arow = A + (F.row_ofs[f] + 3 * (int64_t)a) * lda;
    const int tid = threadIdx.x;

    for (int64_t c0 = e0; c0 < e1; c0 += MB_MAX_ENT) {
        const int nent = (int)min((int64_t)MB_MAX_ENT, e1 - c0);
        sort_incidences<NBODY>(CS, inc, revs, typ, N, qbase, c0, nent, nkeys, sEnt, sKey, sOrd, sCnt);
        for (int T = 0; T < ntypes; ++T) {
            const int gbeg = T == 0 ? 0 : sCnt[T * 4 - 1], gend = sCnt[T * 4 + 3];
            const ClusterTypeDev& CT = types[T];
            const int n = CT.n_allowed;
            if (gbeg == gend || n == 0) continue;
            const int S = (n + NT - 1) / NT;                   // powers per thread
            const int pb = min(n, tid * S), pe = min(n, pb + S);
            const int tb = CT.pow_offset / NP;                 // the type's first power in offs / tcol
            R* const acol = arow + CT.col_base;
            // the thread's first column began in an earlier thread's range
            const bool head = pb < pe && pb > 0 && tcol[tb + pb - 1] == tcol[tb + pb];
            for (int ch0 = gbeg; ch0 < gend; ch0 += CB) {
                const int nb = min(CB, gend - ch0);
                const bool add = !single_pass || ch0 > gbeg;   // later chunks add to the rows
                if (tid < nb) {
                    const int k = sOrd[ch0 + tid];
                    const int v = sEnt[k];
                    sQ[tid] = v >> 2; sM[tid] = v & 3; sRole[tid] = sKey[k] & 3;
                    if (pre) {
                        const int4 mm = CS.m[qbase + (v >> 2)];
                        int id = 0, w = 1;
                        for (int u = 0; u < NBODY; ++u) { id += w * (typ[member(mm, u) % N] + 1); w *= 10; }
                        for (int s = 0; s < NP; ++s) {
                            int ea, eb;
                            slot_edge(M, NBODY, id, s, ea, eb);
                            sSg[tid * NP + s] = ((v & 3) == ea) ? 1 : (((v & 3) == eb) ? -1 : 0);
                        }
                    }
                }
                __syncthreads();
                // (1) per (cluster, slot): basis and the owner's weighted derivative
                if (pre) {
                    const int stride = 2 * ord + 4;
                    for (int t = tid; t < nb * NP; t += NT) {
                        const int c = t / NP, s = t % NP;
                        const R* src = pre + ((size_t)(qbase + sQ[c]) * NP + s) * stride;
                        const int sg = sSg[c * NP + s];
                        const R ir = sg != 0 ? R(sg) / src[2 * ord] : R(0);   // sign / r in the form's type
                        const R wx = src[2 * ord + 1] * ir, wy = src[2 * ord + 2] * ir, wz = src[2 * ord + 3] * ir;
                        R* g = sGH + ((size_t)c * NP + s) * 2 * ord;
                        R* hw = sW + ((size_t)c * NP + s) * 3 * ord;
                        for (int j = 0; j < ord; ++j) {
                            const R gn = src[j], hn = src[ord + j];
                            g[j] = gn; g[ord + j] = hn;
                            hw[j] = hn * wx; hw[ord + j] = hn * wy; hw[2 * ord + j] = hn * wz;
                        }
                    }
                } else
                for (int t = tid; t < nb * NP; t += NT) {
                    const int c = t / NP, s = t % NP;
                    const int4 mm = CS.m[qbase + sQ[c]];
                    int id = 0, w = 1;
                    for (int u = 0; u < NBODY; ++u) { id += w * (typ[member(mm, u) % N] + 1); w *= 10; }
                    SlotBasis sb;
                    R* g = sGH + ((size_t)c * NP + s) * 2 * ord;
                    slot_basis<R>(M, F, NBODY, f, mm, id, T, s, ord, g, g + ord, sb);
                    const int m = sM[c];
                    const double sg = (m == sb.ma) ? 1.0 : ((m == sb.mb) ? -1.0 : 0.0);
                    const double ir = sg / sb.r;
                    const R wx = R(sb.rab[0] * ir), wy = R(sb.rab[1] * ir), wz = R(sb.rab[2] * ir);
                    R* hw = sW + ((size_t)c * NP + s) * 3 * ord;
                    const R* h = g + ord;
                    for (int j = 0; j < ord; ++j) { hw[j] = h[j] * wx; hw[ord + j] = h[j] * wy; hw[2 * ord + j] = h[j] * wz; }
                }
                __syncthreads();
                // (2) M_x,y,z over the incident-slot powers, Q (times PERM_SCALE) over
                // the others, each cluster with its owner's role.  4-body M items cover
                // one (p0, p1) pair and every p2:
                //   M[p0,p1,p2] = (w0 h0 g1 + g0 w1 h1)[p0,p1] g2[p2] + (g0 g1)[p0,p1] w2 h2[p2]
                const int nzm = NI == 3 ? ord * ord : sizeI;   // M items per cluster
                const int nzt = nzm + sizeO;
                for (int t = tid; t < nb * nzt; t += NT) {
                    const int c = t / nzt, z = t % nzt;
                    const int role = sRole[c];
                    const R* GH = sGH + (size_t)c * NP * 2 * ord;
                    const R* HW = sW + (size_t)c * NP * 3 * ord;
                    R* tab = sTab + (size_t)c * per;
                    if (z < nzm) {
                        const int p0 = z % ord, p1 = z / ord % ord;
                        const R* g0 = GH + (size_t)role_slot_in(NBODY, role, 0) * 2 * ord;
                        const R* g1 = GH + (size_t)role_slot_in(NBODY, role, 1) * 2 * ord;
                        const R* w0 = HW + (size_t)role_slot_in(NBODY, role, 0) * 3 * ord;
                        const R* w1 = HW + (size_t)role_slot_in(NBODY, role, 1) * 3 * ord;
                        if constexpr (NI == 2) {
                            tab[z] = w0[p0] * g1[p1] + w1[p1] * g0[p0];
                            tab[sizeI + z] = w0[ord + p0] * g1[p1] + w1[ord + p1] * g0[p0];
                            tab[2 * sizeI + z] = w0[2 * ord + p0] * g1[p1] + w1[2 * ord + p1] * g0[p0];
                        } else {
                            const R* g2 = GH + (size_t)role_slot_in(NBODY, role, 2) * 2 * ord;
                            const R* w2 = HW + (size_t)role_slot_in(NBODY, role, 2) * 3 * ord;
                            const R a0 = g0[p0], a1 = g1[p1];
                            const R gg = a0 * a1;
                            const R bx = w0[p0] * a1 + a0 * w1[p1];
                            const R by = w0[ord + p0] * a1 + a0 * w1[ord + p1];
                            const R bz = w0[2 * ord + p0] * a1 + a0 * w1[2 * ord + p1];
                            for (int p2 = 0; p2 < ord; ++p2) {
                                const int zz = z + p2 * ord * ord;
                                const R c2 = g2[p2];
                                tab[zz] = bx * c2 + gg * w2[p2];
                                tab[sizeI + zz] = by * c2 + gg * w2[ord + p2];
                                tab[2 * sizeI + zz] = bz * c2 + gg * w2[2 * ord + p2];
                            }
                        }
                    } else {
                        int zz = z - nzm;
                        R prod = R(perm);
                        for (int u = 0; u < NO; ++u) {
                            prod *= GH[(size_t)role_slot_out(NBODY, role, u) * 2 * ord + zz % ord];
                            zz /= ord;
                        }
                        tab[3 * sizeI + (z - nzm)] = prod;
                    }
                }
                __syncthreads();
                // (3) the thread's powers: 3 FMAs per (power, cluster), summed per column
                int rs[NBODY], re[NBODY];   // each role's clusters within the chunk
#pragma unroll
                for (int r = 0; r < NBODY; ++r) {
                    const int key = T * 4 + r;
                    rs[r] = max(key == 0 ? 0 : sCnt[key - 1], ch0) - ch0;
                    re[r] = min(sCnt[key], ch0 + nb) - ch0;
                }
                auto put = [&](int col, R x, R y, R z) {
                    R* p0 = acol + col;
                    if (add) { p0[0] += x; p0[lda] += y; p0[2 * lda] += z; }
                    else { p0[0] = x; p0[lda] = y; p0[2 * lda] = z; }
                };
                R ax = R(0), ay = R(0), az = R(0);
                int pcol = -1;
                bool first = true;   // still in the thread's first column
                for (int p = pb; p < pe; ++p) {
                    const int col = tcol[tb + p];
                    if (p > pb && col != pcol) {   // column pcol ended at p - 1
                        if (first && head) { sPart[3 * tid] = ax; sPart[3 * tid + 1] = ay; sPart[3 * tid + 2] = az; }
                        else put(pcol, ax, ay, az);
                        first = false;
                        ax = ay = az = R(0);
                    }
                    pcol = col;
                    const uint4 o4 = offs[tb + p];
                    const uint32_t ow[4] = {o4.x, o4.y, o4.z, o4.w};
#pragma unroll
                    for (int r = 0; r < NBODY; ++r) {
                        const int oM = (int)(ow[r] & 0xffffu), oQ = (int)(ow[r] >> 16);
                        for (int c = rs[r]; c < re[r]; ++c) {
                            const R* tab = sTab + (size_t)c * per;
                            const R qv = tab[oQ];
                            ax += tab[oM] * qv; ay += tab[sizeI + oM] * qv; az += tab[2 * sizeI + oM] * qv;
                        }
                    }
                }
                bool tail = false;   // the last column continues into later ranges
                if (pb < pe) {
                    const bool ends = pe == n || tcol[tb + pe] != pcol;
                    if (first && head) { sPart[3 * tid] = ax; sPart[3 * tid + 1] = ay; sPart[3 * tid + 2] = az; }
                    else if (ends) put(pcol, ax, ay, az);
                    else tail = true;
                }
                __syncthreads();
                if (tail) {   // add the later ranges' partials of this column in thread order
                    const int last = (grps[CT.grp_offset + pcol + 1] - 1) / S;
                    for (int t2 = tid + 1; t2 <= last; ++t2) {
                        ax += sPart[3 * t2]; ay += sPart[3 * t2 + 1]; az += sPart[3 * t2 + 2];
                    }
                    put(pcol, ax, ay, az);
                }
            }
        }
    }
}

// ---------------------------------------------------------------- many-body stress/energy rows
// grid: (frame, cluster type, group-aligned power chunk); comps as in k_virial2.
// grid: x = frame * ntypes + type, y = group-aligned power chunk, z = cluster chunk.
// Each CTA sums VIR_CLUSTERS clusters and stores its column partials (7 comps);
// k_virial_reduce adds the chunks in order and writes the rows.
template <int NBODY, typename R, int PPT>
__global__ void __launch_bounds__(MB_THREADS, (PPT == 1 && sizeof(R) == 4) ? 2 : 1) k_virial_mb(ModelDev M, FramesDev F, ClusterSet CS, Buckets bytype,
                                                          const int64_t* key_frame_ofs, int ncomp,
                                                          const R* __restrict__ pre, R* part,
                                                          int ntrue_max, int nchunks_max) {
    constexpr int NP = NBODY == 3 ? 3 : 6;
    constexpr int N1 = NBODY - 1;
    constexpr int N2 = NP - N1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ntypes = NBODY == 3 ? M.ntypes3 : M.ntypes4;
    const int f = blockIdx.x / ntypes;
    const int T = blockIdx.x % ntypes;
    const int srows = F.stress_rows[f], erows = F.energy_rows[f];
    if (srows == 0 && erows == 0) return;
    const ClusterTypeDev& CT = (NBODY == 3 ? M.types3 : M.types4)[T];
    if ((int)blockIdx.y >= CT.vir_nchunk) return;
    const int pbeg = CT.vir_chunk[blockIdx.y], pend = CT.vir_chunk[blockIdx.y + 1];
    const int64_t kb = key_frame_ofs[f];
    const int64_t t0 = bytype.key_ofs[kb + T], t1 = bytype.key_ofs[kb + T + 1];
    const int64_t c0 = t0 + (int64_t)blockIdx.z * VIR_CLUSTERS;
    if (c0 >= t1) return;
    const int64_t c1 = min(t1, c0 + (int64_t)VIR_CLUSTERS);
    const int ord = NBODY == 3 ? M.order3 : M.order4;
    const uint8_t* pows = NBODY == 3 ? M.pow3 : M.pow4;
    const int* grps = NBODY == 3 ? M.grp3 : M.grp4;
    const int N = F.natoms[f];
    const BoxDev& B = F.box[f];
    const double perm = NBODY == 3 ? B.perm3 : B.perm4;
    const int64_t qbase = CS.ofs[F.atom_ofs[f]];
    const int* typ = F.type + F.atom_ofs[f];
    int size1 = 1, size2 = 1;
    for (int k = 0; k < N1; ++k) size1 *= ord;
    for (int k = 0; k < N2; ++k) size2 *= ord;
    const int per = 7 * size1 + 7 * size2;   // [Q1 | A1 xx..yz | Q2 | A2 xx..yz]
    int S1[3], S2[3];
    role_slots(NBODY, 0, S1, S2);
    const MbVirSmem L = mb_vir_smem(NBODY, ord, PPT * MB_THREADS, (int)sizeof(R));
    int* sQ = reinterpret_cast<int*>(smem_raw + L.q);
    R* sGH = reinterpret_cast<R*>(smem_raw + L.gh);
    R* sV = reinterpret_cast<R*>(smem_raw + L.v);
    R* sTab = reinterpret_cast<R*>(smem_raw + L.tab);

    int i1[PPT], i2[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const int p = pbeg + threadIdx.x + k * blockDim.x;
        i1[k] = -1; i2[k] = 0;
        if (p < pend) {
            const uint8_t* pw = pows + CT.pow_offset + (size_t)p * NP;
            int x = 0, y = 0;
            for (int t = N1 - 1; t >= 0; --t) x = x * ord + pw[S1[t]];
            for (int t = N2 - 1; t >= 0; --t) y = y * ord + pw[S2[t]];
            i1[k] = x; i2[k] = y;
        }
    }
    R acc[PPT][7];
#pragma unroll
    for (int k = 0; k < PPT; ++k)
        for (int c = 0; c < 7; ++c) acc[k][c] = R(0);
    for (int64_t b0 = c0; b0 < c1; b0 += MB_CB) {
        const int nb = (int)min((int64_t)MB_CB, c1 - b0);
        if (threadIdx.x < nb) sQ[threadIdx.x] = bytype.val[b0 + threadIdx.x];
        __syncthreads();
        if (pre) {   // bases of the cluster tables, one thread per (cluster, slot, power)
            const int stride = 2 * ord + 4;
            for (int t = threadIdx.x; t < nb * NP * ord; t += blockDim.x) {
                const int c = t / (NP * ord), rem = t % (NP * ord), s = rem / ord, n = rem % ord;
                const R* src = pre + ((size_t)(qbase + sQ[c]) * NP + s) * stride;
                R* g = sGH + ((size_t)c * NP + s) * 2 * ord;
                g[n] = src[n]; g[ord + n] = src[ord + n];
                if (n == 0) {   // r_a r_b / r in the form's type
                    const R r = src[2 * ord];
                    const R x[3] = {src[2 * ord + 1], src[2 * ord + 2], src[2 * ord + 3]};
                    R* v = sV + ((size_t)c * NP + s) * 6;
                    v[0] = x[0] * x[0] / r; v[1] = x[1] * x[1] / r; v[2] = x[2] * x[2] / r;
                    v[3] = x[0] * x[1] / r; v[4] = x[0] * x[2] / r; v[5] = x[1] * x[2] / r;
                }
            }
        } else
        for (int t = threadIdx.x; t < nb * NP; t += blockDim.x) {
            const int c = t / NP, s = t % NP;
            const int4 mm = CS.m[qbase + sQ[c]];
            int id = 0, w = 1;
            for (int u = 0; u < NBODY; ++u) { id += w * (typ[member(mm, u) % N] + 1); w *= 10; }
            SlotBasis sb;
            R* g = sGH + ((size_t)c * NP + s) * 2 * ord;
            slot_basis<R>(M, F, NBODY, f, mm, id, T, s, ord, g, g + ord, sb);
            R* v = sV + ((size_t)c * NP + s) * 6;
            const double* x = sb.rab;
            v[0] = R(x[0] * x[0] / sb.r); v[1] = R(x[1] * x[1] / sb.r); v[2] = R(x[2] * x[2] / sb.r);
            v[3] = R(x[0] * x[1] / sb.r); v[4] = R(x[0] * x[2] / sb.r); v[5] = R(x[1] * x[2] / sb.r);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < nb * (size1 + size2); t += blockDim.x) {
            const int c = t / (size1 + size2);
            int z = t % (size1 + size2);
            const bool first = z < size1;
            const int* S = first ? S1 : S2;
            const int ns = first ? N1 : N2;
            if (!first) z -= size1;
            const R* GH = sGH + (size_t)c * NP * 2 * ord;
            const R* V = sV + (size_t)c * NP * 6;
            int pwr[3] = {0, 0, 0}, zz = z;
            for (int u = 0; u < ns; ++u) { pwr[u] = zz % ord; zz /= ord; }
            R q = R(1), av[6] = {0, 0, 0, 0, 0, 0};
            for (int u = 0; u < ns; ++u) q *= GH[(size_t)S[u] * 2 * ord + pwr[u]];
            for (int u = 0; u < ns; ++u) {
                R prod = GH[(size_t)S[u] * 2 * ord + ord + pwr[u]];
                for (int v2 = 0; v2 < ns; ++v2) if (v2 != u) prod *= GH[(size_t)S[v2] * 2 * ord + pwr[v2]];
                for (int k = 0; k < 6; ++k) av[k] += prod * V[S[u] * 6 + k];
            }
            R* tab = sTab + (size_t)c * per + (first ? 0 : 7 * size1);
            const int sz = first ? size1 : size2;
            tab[z] = q;
            for (int k = 0; k < 6; ++k) tab[(1 + k) * sz + z] = av[k];
        }
        __syncthreads();
        for (int c = 0; c < nb; ++c) {
            const R* t1 = sTab + (size_t)c * per;
            const R* t2 = t1 + 7 * size1;
#pragma unroll
            for (int k = 0; k < PPT; ++k) {
                if (i1[k] < 0) continue;
                const R q1 = t1[i1[k]], q2 = t2[i2[k]];
                acc[k][0] = fma(q1, q2, acc[k][0]);
#pragma unroll
                for (int cc = 1; cc < 7; ++cc) {   // fully unrolled: accumulators stay in registers
                    if (cc < ncomp) {
                        acc[k][cc] = fma(-t1[cc * size1 + i1[k]], q2, acc[k][cc]);
                        acc[k][cc] = fma(-q1, t2[cc * size2 + i2[k]], acc[k][cc]);
                    }
                }
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const int pl = threadIdx.x + k * blockDim.x;
        if (pbeg + pl < pend)
            for (int c = 0; c < 7; ++c) sTab[(size_t)pl * 7 + c] = acc[k][c];
    }
    __syncthreads();
    const int* gp = grps + CT.grp_offset;
    R* out = part + ((size_t)blockIdx.x * nchunks_max + blockIdx.z) * 7 * ntrue_max;
    for (int col = threadIdx.x; col < CT.n_true; col += blockDim.x) {
        const int pa = gp[col], pb = gp[col + 1];
        if (pa < pbeg || pa >= pend) continue;
        R sv[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int p = pa; p < pb; ++p)
            for (int c = 0; c < 7; ++c) sv[c] += sTab[(size_t)(p - pbeg) * 7 + c];
        for (int c = 0; c < 7; ++c) out[(size_t)c * ntrue_max + col] = sv[c];
    }
}

// Sum the cluster-chunk partials of each (frame, type) in chunk order and write the
// stress / energy rows (PERM_SCALE and 1/V applied once, at the end).
template <int NBODY, typename R>
__global__ void k_virial_reduce(ModelDev M, FramesDev F, Buckets bytype, const int64_t* key_frame_ofs,
                                const R* part, int ntrue_max, int nchunks_max, R* A, int64_t lda) {
    const int ntypes = NBODY == 3 ? M.ntypes3 : M.ntypes4;
    const int f = blockIdx.x / ntypes;
    const int T = blockIdx.x % ntypes;
    if (F.stress_rows[f] == 0 && F.energy_rows[f] == 0) return;
    const ClusterTypeDev& CT = (NBODY == 3 ? M.types3 : M.types4)[T];
    const int64_t kb = key_frame_ofs[f];
    const int64_t n = bytype.key_ofs[kb + T + 1] - bytype.key_ofs[kb + T];
    if (n == 0) return;
    const int nch = (int)((n + VIR_CLUSTERS - 1) / VIR_CLUSTERS);
    const BoxDev& B = F.box[f];
    const double perm = NBODY == 3 ? B.perm3 : B.perm4;
    const double inv_vol = 1.0 / B.vol;
    const R* base = part + (size_t)blockIdx.x * nchunks_max * 7 * ntrue_max;
    for (int col = threadIdx.x; col < CT.n_true; col += blockDim.x) {
        R sv[7] = {0, 0, 0, 0, 0, 0, 0};
        for (int c = 0; c < nch; ++c)
            for (int k = 0; k < 7; ++k) sv[k] += base[((size_t)c * 7 + k) * ntrue_max + col];
        for (int k = 0; k < 7; ++k) sv[k] = R(sv[k] * perm);
        write_virial_rows(F, f, CT.col_base + col, sv, inv_vol, A, lda);
    }
}

// Largest cluster count of any (frame, type) bucket.
__global__ void k_max_bucket(const int64_t* key_ofs, const int64_t* key_frame_ofs, int nframes, int ntypes,
                             int* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nframes * ntypes) return;
    const int f = i / ntypes, T = i % ntypes;
    const int64_t kb = key_frame_ofs[f];
    atomicMax(out, (int)(key_ofs[kb + T + 1] - key_ofs[kb + T]));
}

// ---------------------------------------------------------------- energy offset columns
// One column per atom type holding that type's atom count on energy rows
// (A_MAT::add_col_of_ones src/A_Matrix.C:155-175); force and stress rows keep 0.
// HIERARC-excluded types have no column.
__global__ void k_energy_cols(ModelDev M, FramesDev F, void* A, int64_t lda, int is_double) {
    const int f = blockIdx.x;
    if (F.energy_rows[f] == 0 || M.fit_ener_cols == 0) return;
    const int N = F.natoms[f];
    const int* typ = F.type + F.atom_ofs[f];
    const int64_t row = F.row_ofs[f] + 3 * (int64_t)N + F.stress_rows[f];
    for (int t = threadIdx.x; t < M.fit_ener_cols; t += blockDim.x) {
        if (M.ener_col[t] < 0) continue;   // HIERARC EXCLUDE 1B: no column
        int count = 0;
        for (int k = 0; k < N; ++k) count += typ[k] == t;
        for (int rr = 0; rr < F.energy_rows[f]; ++rr) {
            const int64_t idx = (row + rr) * lda + M.tot_short + M.ncoul + M.ener_col[t];
            if (is_double) reinterpret_cast<double*>(A)[idx] = (double)count;
            else reinterpret_cast<float*>(A)[idx] = (float)count;
        }
    }
}

// ---------------------------------------------------------------- launchers
template <typename K>
static void set_smem(K kernel, size_t bytes) {
    if (bytes > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

void launch_force2(int prec, int nreal, const ModelDev& M, const FramesDev& F, const NeighDev& NB,
                   const Buckets& inc, const int64_t* kfo, void* A, int64_t lda, cudaStream_t st) {
    const size_t rs = prec == 0 ? 8 : 4;
    const size_t sm = (size_t)F2_THREADS * 3 * M.order2 * rs + F2_THREADS * sizeof(int);
    if (prec == 0) {
        set_smem(k_force2<double>, sm);
        k_force2<double><<<nreal, F2_THREADS, sm, st>>>(M, F, NB, inc, kfo, (double*)A, lda);
    } else {
        set_smem(k_force2<float>, sm);
        k_force2<float><<<nreal, F2_THREADS, sm, st>>>(M, F, NB, inc, kfo, (float*)A, lda);
    }
}

int virial2_slices(int nframes, int64_t npairs, int sms) {
    if (nframes <= 0) return 1;
    const int64_t per_frame = npairs / nframes;
    const int64_t want = (2 * (int64_t)sms + nframes - 1) / nframes;       // about two CTAs per SM
    const int64_t most = std::max<int64_t>(1, per_frame / (2 * F2_THREADS));   // two chunks of pairs per slice
    return (int)std::max<int64_t>(1, std::min<int64_t>({want, most, 64}));
}

template <typename R, int MAXC>
static void virial2_launch(int nframes, int nslice, size_t sm, const ModelDev& M, const FramesDev& F,
                           const NeighDev& NB, void* part, void* A, int64_t lda, cudaStream_t st) {
    set_smem(k_virial2<R, MAXC>, sm);
    k_virial2<R, MAXC><<<dim3((unsigned)nframes, (unsigned)nslice), F2_THREADS, sm, st>>>(M, F, NB, nslice, (R*)part);
    k_virial2_rows<R><<<nframes, F2_THREADS, 0, st>>>(M, F, nslice, (const R*)part, (R*)A, lda);
}

template <typename R>
static void virial2_dispatch(int maxc, int nframes, int nslice, size_t sm, const ModelDev& M, const FramesDev& F,
                             const NeighDev& NB, void* part, void* A, int64_t lda, cudaStream_t st) {
    if (maxc <= 1) virial2_launch<R, 1>(nframes, nslice, sm, M, F, NB, part, A, lda, st);
    else if (maxc <= 2) virial2_launch<R, 2>(nframes, nslice, sm, M, F, NB, part, A, lda, st);
    else if (maxc <= 4) virial2_launch<R, 4>(nframes, nslice, sm, M, F, NB, part, A, lda, st);
    else virial2_launch<R, 8>(nframes, nslice, sm, M, F, NB, part, A, lda, st);
}

void launch_virial2(int prec, int nframes, int nslice, const ModelDev& M, const FramesDev& F, const NeighDev& NB,
                    void* part, void* A, int64_t lda, cudaStream_t st) {
    if (nframes <= 0) return;
    const size_t rs = prec == 0 ? 8 : 4;
    const size_t sm = (size_t)F2_THREADS * (2 * M.order2 + 6) * rs + F2_THREADS * sizeof(int);
    const int maxc = (M.npairs * M.order2 + F2_THREADS - 1) / F2_THREADS;   // at most 8 (checked by the caller)
    if (prec == 0) virial2_dispatch<double>(maxc, nframes, nslice, sm, M, F, NB, part, A, lda, st);
    else virial2_dispatch<float>(maxc, nframes, nslice, sm, M, F, NB, part, A, lda, st);
}

size_t cluster_basis_count(int nbody, int ord, int64_t nclusters) {
    return (size_t)nclusters * (nbody == 3 ? 3 : 6) * (2 * ord + 4);
}

void launch_cluster_basis(int nbody, int prec, int64_t nq, const ModelDev& M, const FramesDev& F,
                          const ClusterSet& CS, void* basis, cudaStream_t st) {
    const int64_t n = nq * (nbody == 3 ? 3 : 6);
    if (n == 0) return;
    const unsigned blocks = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 64);
    if (nbody == 3 && prec == 0) k_cluster_basis<3, double><<<blocks, 256, 0, st>>>(M, F, CS, nq, (double*)basis);
    else if (nbody == 3) k_cluster_basis<3, float><<<blocks, 256, 0, st>>>(M, F, CS, nq, (float*)basis);
    else if (prec == 0) k_cluster_basis<4, double><<<blocks, 256, 0, st>>>(M, F, CS, nq, (double*)basis);
    else k_cluster_basis<4, float><<<blocks, 256, 0, st>>>(M, F, CS, nq, (float*)basis);
}

template <int NBD, typename R>
static void force_mb_ppt(int ppt, int nreal, size_t smem, const ModelDev& M, const FramesDev& F, const ClusterSet& CS,
                         const Buckets& inc, const int64_t* kfo, const R* pre, R* A, int64_t lda, cudaStream_t st,
                         int nt4) {
    if (ppt <= 1) {
        set_smem(k_force_mb<NBD, R, 1>, smem);
        k_force_mb<NBD, R, 1><<<nreal, MB_THREADS, smem, st>>>(M, F, CS, inc, kfo, pre, A, lda);
    } else if (ppt <= 2) {
        set_smem(k_force_mb<NBD, R, 2>, smem);
        k_force_mb<NBD, R, 2><<<nreal, MB_THREADS, smem, st>>>(M, F, CS, inc, kfo, pre, A, lda);
    } else if (NBD == 4 && nt4 == 2 * MB_THREADS) {   // up to 8 powers per thread at MB_THREADS = 4 at twice the threads
        set_smem(k_force_mb<NBD, R, 4, 2 * MB_THREADS>, smem);
        k_force_mb<NBD, R, 4, 2 * MB_THREADS><<<nreal, 2 * MB_THREADS, smem, st>>>(M, F, CS, inc, kfo, pre, A, lda);
    } else {
        set_smem(k_force_mb<NBD, R, 8>, smem);
        k_force_mb<NBD, R, 8><<<nreal, MB_THREADS, smem, st>>>(M, F, CS, inc, kfo, pre, A, lda);
    }
}

template <int NBD, typename R>
static void force_rg(int nreal, int nt, size_t smem, const ModelDev& M, const FramesDev& F, const ClusterSet& CS,
                     const Buckets& inc, const int64_t* kfo, const R* pre, R* A, int64_t lda, cudaStream_t st) {
    set_smem(k_force_rg<NBD, R>, smem);
    k_force_rg<NBD, R><<<nreal, nt, smem, st>>>(M, F, CS, inc, kfo, pre, A, lda);
}

int rg_threads(const int* n_allowed, int ntypes, int rsize) {
    const int mx = rg_max_threads(rsize);
    if (rsize != 8) return mx;
    int best = mx;
    long long best_idle = -1;
    for (int nt = mx; nt >= mx / 2; nt -= 32) {
        long long idle = 0;
        for (int t = 0; t < ntypes; ++t) {
            const int n = n_allowed[t];
            if (n > 0) idle += (long long)((n + nt - 1) / nt) * nt - n;
        }
        if (best_idle < 0 || idle < best_idle) { best_idle = idle; best = nt; }
    }
    return best;
}

void launch_force_rg(int nbody, int prec, int nreal, int nt, size_t smem, const ModelDev& M, const FramesDev& F,
                     const ClusterSet& CS, const Buckets& inc, const int64_t* kfo, const void* pre, void* A,
                     int64_t lda, cudaStream_t st) {
    if (nbody == 3 && prec == 0)
        force_rg<3, double>(nreal, nt, smem, M, F, CS, inc, kfo, (const double*)pre, (double*)A, lda, st);
    else if (nbody == 3)
        force_rg<3, float>(nreal, nt, smem, M, F, CS, inc, kfo, (const float*)pre, (float*)A, lda, st);
    else if (prec == 0)
        force_rg<4, double>(nreal, nt, smem, M, F, CS, inc, kfo, (const double*)pre, (double*)A, lda, st);
    else
        force_rg<4, float>(nreal, nt, smem, M, F, CS, inc, kfo, (const float*)pre, (float*)A, lda, st);
}

void launch_force_mb(int nbody, int prec, int ppt, int nreal, size_t smem, const ModelDev& M, const FramesDev& F,
                     const ClusterSet& CS, const Buckets& inc, const int64_t* kfo, const void* pre, void* A,
                     int64_t lda, cudaStream_t st, int nt4) {
    if (nbody == 3 && prec == 0)
        force_mb_ppt<3, double>(ppt, nreal, smem, M, F, CS, inc, kfo, (const double*)pre, (double*)A, lda, st, nt4);
    else if (nbody == 3)
        force_mb_ppt<3, float>(ppt, nreal, smem, M, F, CS, inc, kfo, (const float*)pre, (float*)A, lda, st, nt4);
    else if (prec == 0)
        force_mb_ppt<4, double>(ppt, nreal, smem, M, F, CS, inc, kfo, (const double*)pre, (double*)A, lda, st, nt4);
    else
        force_mb_ppt<4, float>(ppt, nreal, smem, M, F, CS, inc, kfo, (const float*)pre, (float*)A, lda, st, nt4);
}

template <int NBD, typename R, int PPT>
static void virial_mb_ppt(dim3 grid, unsigned rgrid, size_t smem, const ModelDev& M, const FramesDev& F,
                          const ClusterSet& CS, const Buckets& byt, const int64_t* kfo, int ncomp, const R* pre,
                          R* part, int ntrue_max, int nchunks_max, R* A, int64_t lda, cudaStream_t st) {
    set_smem(k_virial_mb<NBD, R, PPT>, smem);
    k_virial_mb<NBD, R, PPT><<<grid, MB_THREADS, smem, st>>>(M, F, CS, byt, kfo, ncomp, pre, part, ntrue_max,
                                                              nchunks_max);
    k_virial_reduce<NBD, R><<<rgrid, 256, 0, st>>>(M, F, byt, kfo, part, ntrue_max, nchunks_max, A, lda);
}

template <int NBD, typename R>
static void virial_mb_typed(int ppt, dim3 grid, unsigned rgrid, size_t smem, const ModelDev& M, const FramesDev& F,
                            const ClusterSet& CS, const Buckets& byt, const int64_t* kfo, int ncomp, const void* pre,
                            void* part, int ntrue_max, int nchunks_max, void* A, int64_t lda, cudaStream_t st) {
    if (ppt == 1)
        virial_mb_ppt<NBD, R, 1>(grid, rgrid, smem, M, F, CS, byt, kfo, ncomp, (const R*)pre, (R*)part, ntrue_max,
                                 nchunks_max, (R*)A, lda, st);
    else
        virial_mb_ppt<NBD, R, VIR_PPT>(grid, rgrid, smem, M, F, CS, byt, kfo, ncomp, (const R*)pre, (R*)part,
                                       ntrue_max, nchunks_max, (R*)A, lda, st);
}

void launch_virial_mb(int nbody, int prec, int ppt, int nframes, int ntypes, int nzchunk, int nchunks_max,
                      int ntrue_max, size_t smem, const ModelDev& M, const FramesDev& F, const ClusterSet& CS,
                      const Buckets& byt, const int64_t* kfo, int ncomp, const void* pre, void* part, void* A,
                      int64_t lda, cudaStream_t st) {
    dim3 grid(nframes * ntypes, nzchunk, nchunks_max);
    const unsigned rgrid = (unsigned)(nframes * ntypes);
    if (nbody == 3 && prec == 0)
        virial_mb_typed<3, double>(ppt, grid, rgrid, smem, M, F, CS, byt, kfo, ncomp, pre, part, ntrue_max,
                                   nchunks_max, A, lda, st);
    else if (nbody == 3)
        virial_mb_typed<3, float>(ppt, grid, rgrid, smem, M, F, CS, byt, kfo, ncomp, pre, part, ntrue_max,
                                  nchunks_max, A, lda, st);
    else if (prec == 0)
        virial_mb_typed<4, double>(ppt, grid, rgrid, smem, M, F, CS, byt, kfo, ncomp, pre, part, ntrue_max,
                                   nchunks_max, A, lda, st);
    else
        virial_mb_typed<4, float>(ppt, grid, rgrid, smem, M, F, CS, byt, kfo, ncomp, pre, part, ntrue_max,
                                  nchunks_max, A, lda, st);
}

void launch_max_bucket(const int64_t* key_ofs, const int64_t* kfo, int nframes, int ntypes, int* out,
                       cudaStream_t st) {
    const int n = nframes * ntypes;
    if (n > 0) k_max_bucket<<<(n + 255) / 256, 256, 0, st>>>(key_ofs, kfo, nframes, ntypes, out);
}

void launch_energy_cols(int prec, int nframes, const ModelDev& M, const FramesDev& F, void* A, int64_t lda,
                        cudaStream_t st) {
    k_energy_cols<<<nframes, 32, 0, st>>>(M, F, A, lda, prec == 0 ? 1 : 0);
}

}  // namespace cgd
