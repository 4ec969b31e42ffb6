// Geometry, neighbour lists and cluster enumeration on the device.
//
// Reference behaviour reproduced here (all index sets are bit-exact):
//   FRAME::build_layers / update_ghost  src/ClassDefs.C:2361-2409, 2685-2752
//   BOX::WRAP_ATOM / LAYER_ATOM          src/ClassDefs.C:2064-2164
//   NEIGHBORS::DO_UPDATE_BIG / _SMALL    src/ClassDefs.C:137-393
//   triplet loops of Cheby::Deriv_3B     src/Cheby.C:981-1054
//   quadruplet loops of Cheby::Deriv_4B  src/Cheby.C:1387-1500
//   FCUT::PROCEED                        src/Fcut.C:125-140
// The reference decides membership with FP64 distances; every candidate is first
// screened with an FP32 distance (margin 1e-2 A, far above FP32 error) and only
// candidates near a cut-off are re-decided with the exact FP64 sequence.
#include "dev.cuh"
#include "kernels.h"

namespace cgd {

static constexpr float MARGIN = 1.0e-2f;

// ---------------------------------------------------------------- ghost set-up
__global__ void k_frame_setup(FramesDev F, int64_t total_ghosts) {
    int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= total_ghosts) return;
    // frame lookup: binary search over ghost_ofs
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (F.ghost_ofs[mid] <= gid) lo = mid; else hi = mid - 1;
    }
    const int f = lo;
    const int N = F.natoms[f];
    const int g = (int)(gid - F.ghost_ofs[f]);
    const int a = g % N;
    const int k = g / N;   // 0 = real image
    const BoxDev& B = F.box[f];
    const double* x0 = F.xyz + 3 * (F.atom_ofs[f] + a);
    double w[3];
    // WRAP_ATOM (src/ClassDefs.C:2075-2119); with stored shifts (MD list reuse) the
    // shift of the last list build is applied instead of a fresh floor
    int* sh = (F.shift && F.shift_mode) ? F.shift + 3 * (F.atom_ofs[f] + a) : nullptr;
    const bool use_stored = sh && F.shift_mode == 2;
    const bool store = sh && F.shift_mode == 1 && k == 0;
    if (B.is_ortho) {
        double L3[3] = {B.lx, B.ly, B.lz};
        for (int q = 0; q < 3; ++q) {
            int idx = use_stored ? sh[q] : (int)floor(__ddiv_rn(x0[q], L3[q]));
            if (store) sh[q] = idx;
            w[q] = subrn(x0[q], mulrn((double)idx, L3[q]));
        }
    } else {
        double t[3];
        for (int q = 0; q < 3; ++q) t[q] = dot3rn(B.inv[3 * q], B.inv[3 * q + 1], B.inv[3 * q + 2], x0[0], x0[1], x0[2]);
        for (int q = 0; q < 3; ++q) {
            int idx = use_stored ? sh[q] : (int)floor(t[q]);
            if (store) sh[q] = idx;
            t[q] = subrn(t[q], (double)idx);
        }
        for (int q = 0; q < 3; ++q) w[q] = dot3rn(B.h[3 * q], B.h[3 * q + 1], B.h[3 * q + 2], t[0], t[1], t[2]);
    }
    double c[3] = {w[0], w[1], w[2]};
    if (k > 0) {   // LAYER_ATOM (src/ClassDefs.C:2132-2164)
        int n1, n2, n3;
        layer_index(k - 1, F.nlayers, n1, n2, n3);
        if (B.is_ortho) {
            c[0] = addrn(w[0], mulrn((double)n1, B.h[0]));
            c[1] = addrn(w[1], mulrn((double)n2, B.h[4]));
            c[2] = addrn(w[2], mulrn((double)n3, B.h[8]));
        } else {
            double t[3];
            for (int q = 0; q < 3; ++q) t[q] = dot3rn(B.inv[3 * q], B.inv[3 * q + 1], B.inv[3 * q + 2], w[0], w[1], w[2]);
            t[0] = addrn(t[0], (double)n1); t[1] = addrn(t[1], (double)n2); t[2] = addrn(t[2], (double)n3);
            for (int q = 0; q < 3; ++q) c[q] = dot3rn(B.h[3 * q], B.h[3 * q + 1], B.h[3 * q + 2], t[0], t[1], t[2]);
        }
    }
    double* s = F.scaled + 3 * gid;
    for (int q = 0; q < 3; ++q) s[q] = dot3rn(B.inv[3 * q], B.inv[3 * q + 1], B.inv[3 * q + 2], c[0], c[1], c[2]);
    float4 c32 = make_float4((float)c[0], (float)c[1], (float)c[2], 0.f);
    reinterpret_cast<float4*>(F.cart32)[gid] = c32;
}

// ---------------------------------------------------------------- neighbour lists
// One block of nw warps per real atom (nw = blockDim.x / 32, at most NEIGH_WARPS);
// warp w scans the w-th contiguous slice of the ghost indices, so the concatenated
// lists come out in ghost-index order and the fill pass is deterministic.  With
// several warps the fill pass recounts each slice to place it after the slices
// before it; batches with many atoms use one warp per atom and skip that.
constexpr int NEIGH_WARPS = 8;

__global__ void __launch_bounds__(32 * NEIGH_WARPS) k_neigh(ModelDev M, FramesDev F, NeighDev NB, int fill, int nw) {
    __shared__ int sc[3][NEIGH_WARPS];
    // nw > 1: one atom per block, nw warps on it; nw == 1: one atom per warp
    const int atom = nw > 1 ? blockIdx.x : blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int w = nw > 1 ? threadIdx.x >> 5 : 0;
    const int lane = threadIdx.x & 31;
    if (atom >= NB.n_real) return;
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (F.atom_ofs[mid] <= atom) lo = mid; else hi = mid - 1;
    }
    const int f = lo;
    const int N = F.natoms[f];
    const int i = atom - (int)F.atom_ofs[f];
    const int G = N * F.nimg;
    const int64_t gbase = F.ghost_ofs[f];
    const BoxDev& B = F.box[f];
    const int* typ = F.type + F.atom_ofs[f];
    const int ti = typ[i];
    const float4 ci = reinterpret_cast<const float4*>(F.cart32)[gbase + i];
    const double* si = F.scaled + 3 * (gbase + i);
    const float maxall = (float)fmax(fmax(M.maxcut2, M.order3 > 0 ? M.maxcut3 : 0.0), M.order4 > 0 ? M.maxcut4 : 0.0);
    const float pre = maxall + MARGIN + (float)NB.skin;
    const int per = ((G + nw - 1) / nw + 31) & ~31;
    const int g0 = w * per, g1 = min(G, g0 + per);
    const unsigned lt = (1u << lane) - 1u;
    // bounding box of the frame's real atoms (the first N ghosts); image k of the
    // layers is that box shifted by one lattice translation, so an image whose box lies
    // beyond the search radius of atom i holds none of its neighbours and is skipped
    // (the lists keep their ghost order: only chunks without neighbours are passed over)
    const float4* c32 = reinterpret_cast<const float4*>(F.cart32) + gbase;
    float bmin[3] = {3.0e38f, 3.0e38f, 3.0e38f}, bmax[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
    for (int a = lane; a < N; a += 32) {
        const float4 c = c32[a];
        bmin[0] = fminf(bmin[0], c.x); bmin[1] = fminf(bmin[1], c.y); bmin[2] = fminf(bmin[2], c.z);
        bmax[0] = fmaxf(bmax[0], c.x); bmax[1] = fmaxf(bmax[1], c.y); bmax[2] = fmaxf(bmax[2], c.z);
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int d = 0; d < 3; ++d) {
            bmin[d] = fminf(bmin[d], __shfl_xor_sync(0xffffffffu, bmin[d], o));
            bmax[d] = fmaxf(bmax[d], __shfl_xor_sync(0xffffffffu, bmax[d], o));
        }
    const float reach = pre + 0.05f;   // float rounding of the images' positions stays far below 0.05 A
    const float4 c0 = c32[0];
    auto image_far = [&](int k) {
        const float4 ck = c32[(int64_t)k * N];
        const float s[3] = {ck.x - c0.x, ck.y - c0.y, ck.z - c0.z};
        const float p[3] = {ci.x, ci.y, ci.z};
        float d2 = 0.0f;
        for (int d = 0; d < 3; ++d) {
            const float lo = bmin[d] + s[d], hi = bmax[d] + s[d];
            const float e = p[d] < lo ? lo - p[d] : (p[d] > hi ? p[d] - hi : 0.0f);
            d2 += e * e;
        }
        return d2 > reach * reach;
    };
    auto sweep = [&](bool write, int64_t o2, int64_t o3, int64_t o4, int& c2, int& c3, int& c4) {
        int kseen = -1;
        bool kfar = false;
        for (int base = g0; base < g1;) {
            const int k = base / N;
            if (k != kseen) { kseen = k; kfar = image_far(k); }
            if (kfar) {   // warp-uniform: the rest of image k has no neighbour of atom i
                base = min(g1, (k + 1) * N);
                continue;
            }
            const int g = base + lane;
            base += 32;
            bool in2 = false, in3 = false, in4 = false;
            double r = 0, rab[3] = {0, 0, 0};
            int pt = 0;
            if (g < g1 && g != i && (B.small || i <= g % N)) {
                float4 cg = reinterpret_cast<const float4*>(F.cart32)[gbase + g];
                float dx = cg.x - ci.x, dy = cg.y - ci.y, dz = cg.z - ci.z;
                float r32 = sqrtf(dx * dx + dy * dy + dz * dz);
                if (r32 < pre) {
                    r = dist_exact(B.h, si, F.scaled + 3 * (gbase + g), rab);
                    pt = M.int_pair_map[ti * M.natmtyp + typ[g % N]];
                    const PairDev P = M.pairs[pt];
                    in2 = M.order2 > 0 && r < P.smax + NB.skin && (NB.md || r > P.smin);
                    in3 = M.order3 > 0 && r < M.maxcut3 + NB.skin;
                    in4 = M.order4 > 0 && r < M.maxcut4 + NB.skin;
                }
            }
            const unsigned b2 = __ballot_sync(0xffffffffu, in2);
            const unsigned b3 = __ballot_sync(0xffffffffu, in3);
            const unsigned b4 = __ballot_sync(0xffffffffu, in4);
            if (write) {
                if (in2) {
                    const int64_t p = o2 + c2 + __popc(b2 & lt);
                    NB.i2[p] = i; NB.g2[p] = g; NB.pt2[p] = pt; NB.r2[p] = r;
                    NB.rab2[3 * p] = rab[0]; NB.rab2[3 * p + 1] = rab[1]; NB.rab2[3 * p + 2] = rab[2];
                }
                if (in3) { const int64_t p = o3 + c3 + __popc(b3 & lt); NB.g3[p] = g; NB.r3[p] = r; }
                if (in4) { const int64_t p = o4 + c4 + __popc(b4 & lt); NB.g4[p] = g; NB.r4[p] = r; }
            }
            c2 += __popc(b2); c3 += __popc(b3); c4 += __popc(b4);
        }
    };
    int c2 = 0, c3 = 0, c4 = 0;
    if (nw == 1) {   // single slice per atom: no block-level bookkeeping
        if (fill) {
            sweep(true, NB.ofs2[atom], NB.ofs3[atom], NB.ofs4[atom], c2, c3, c4);
        } else {
            sweep(false, 0, 0, 0, c2, c3, c4);
            if (lane == 0) { NB.cnt2[atom] = c2; NB.cnt3[atom] = c3; NB.cnt4[atom] = c4; }
        }
        return;
    }
    sweep(false, 0, 0, 0, c2, c3, c4);
    if (lane == 0) { sc[0][w] = c2; sc[1][w] = c3; sc[2][w] = c4; }
    __syncthreads();
    if (!fill) {
        if (threadIdx.x == 0) {
            int t2 = 0, t3 = 0, t4 = 0;
            for (int k = 0; k < nw; ++k) { t2 += sc[0][k]; t3 += sc[1][k]; t4 += sc[2][k]; }
            NB.cnt2[atom] = t2; NB.cnt3[atom] = t3; NB.cnt4[atom] = t4;
        }
        return;
    }
    int64_t o2 = NB.ofs2[atom], o3 = NB.ofs3[atom], o4 = NB.ofs4[atom];
    for (int k = 0; k < w; ++k) { o2 += sc[0][k]; o3 += sc[1][k]; o4 += sc[2][k]; }
    int d2 = 0, d3 = 0, d4 = 0;
    sweep(true, o2, o3, o4, d2, d3, d4);
}

// ---------------------------------------------------------------- binned neighbour lists
__device__ __forceinline__ int ghost_frame(const FramesDev& F, int64_t gid) {
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (F.ghost_ofs[mid] <= gid) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int bin_coord(double s, int L, int nb) {
    // s spans [-L, L + 1) over the (2L+1) cell images
    int b = (int)floor((s + L) / (2 * L + 1) * nb);
    return b < 0 ? 0 : (b >= nb ? nb - 1 : b);
}

__device__ __forceinline__ int64_t bin_of(const FramesDev& F, const BinGrid& g, int64_t gid) {
    const double* s = F.scaled + 3 * gid;
    const int L = F.nlayers;
    const int bx = bin_coord(s[0], L, g.nb[0]), by = bin_coord(s[1], L, g.nb[1]), bz = bin_coord(s[2], L, g.nb[2]);
    return g.ofs + ((int64_t)bz * g.nb[1] + by) * g.nb[0] + bx;
}

__global__ void k_bin_count(FramesDev F, int64_t n, Bins B) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= n) return;
    atomicAdd(B.count + bin_of(F, B.grid[ghost_frame(F, gid)], gid), 1);
}

__global__ void k_bin_fill(FramesDev F, int64_t n, Bins B) {
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= n) return;
    const int f = ghost_frame(F, gid);
    const int64_t bin = bin_of(F, B.grid[f], gid);
    const int slot = atomicAdd(B.count + bin, 1);
    B.atoms[B.start[bin] + slot] = (int)(gid - F.ghost_ofs[f]);
}

// One warp per real atom over the ghosts of the 27 bins around it; the per-ghost
// tests are those of k_neigh.
__global__ void __launch_bounds__(256) k_neigh_binned(ModelDev M, FramesDev F, NeighDev NB, Bins BN, int fill) {
    const int atom = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (atom >= NB.n_real) return;
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (F.atom_ofs[mid] <= atom) lo = mid; else hi = mid - 1;
    }
    const int f = lo;
    const int N = F.natoms[f];
    const int i = atom - (int)F.atom_ofs[f];
    const int64_t gbase = F.ghost_ofs[f];
    const BoxDev& B = F.box[f];
    const int* typ = F.type + F.atom_ofs[f];
    const int ti = typ[i];
    const float4 ci = reinterpret_cast<const float4*>(F.cart32)[gbase + i];
    const double* si = F.scaled + 3 * (gbase + i);
    const float maxall = (float)fmax(fmax(M.maxcut2, M.order3 > 0 ? M.maxcut3 : 0.0), M.order4 > 0 ? M.maxcut4 : 0.0);
    const float pre = maxall + MARGIN + (float)NB.skin;
    const BinGrid g = BN.grid[f];
    const int L = F.nlayers;
    const int cx = bin_coord(si[0], L, g.nb[0]), cy = bin_coord(si[1], L, g.nb[1]), cz = bin_coord(si[2], L, g.nb[2]);
    int64_t o2 = 0, o3 = 0, o4 = 0;
    if (fill) { o2 = NB.ofs2[atom]; o3 = NB.ofs3[atom]; o4 = NB.ofs4[atom]; }
    int c2 = 0, c3 = 0, c4 = 0;
    const unsigned lt = (1u << lane) - 1u;
    for (int dz = -1; dz <= 1; ++dz) {
        const int z = cz + dz;
        if (z < 0 || z >= g.nb[2]) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = cy + dy;
            if (y < 0 || y >= g.nb[1]) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int x = cx + dx;
                if (x < 0 || x >= g.nb[0]) continue;
                const int64_t bin = g.ofs + ((int64_t)z * g.nb[1] + y) * g.nb[0] + x;
                const int64_t b0 = BN.start[bin], b1 = BN.start[bin + 1];
                for (int64_t base = b0; base < b1; base += 32) {
                    const int64_t t = base + lane;
                    bool in2 = false, in3 = false, in4 = false;
                    double r = 0, rab[3] = {0, 0, 0};
                    int pt = 0, gg = -1;
                    if (t < b1) {
                        gg = BN.atoms[t];
                        if (gg != i && (B.small || i <= gg % N)) {
                            const float4 cg = reinterpret_cast<const float4*>(F.cart32)[gbase + gg];
                            const float ddx = cg.x - ci.x, ddy = cg.y - ci.y, ddz = cg.z - ci.z;
                            const float r32 = sqrtf(ddx * ddx + ddy * ddy + ddz * ddz);
                            if (r32 < pre) {
                                r = dist_exact(B.h, si, F.scaled + 3 * (gbase + gg), rab);
                                pt = M.int_pair_map[ti * M.natmtyp + typ[gg % N]];
                                const PairDev P = M.pairs[pt];
                                in2 = M.order2 > 0 && r < P.smax + NB.skin && (NB.md || r > P.smin);
                                in3 = M.order3 > 0 && r < M.maxcut3 + NB.skin;
                                in4 = M.order4 > 0 && r < M.maxcut4 + NB.skin;
                            }
                        }
                    }
                    const unsigned b2 = __ballot_sync(0xffffffffu, in2);
                    const unsigned b3 = __ballot_sync(0xffffffffu, in3);
                    const unsigned b4 = __ballot_sync(0xffffffffu, in4);
                    if (fill) {
                        if (in2) {
                            const int64_t p = o2 + c2 + __popc(b2 & lt);
                            NB.i2[p] = i; NB.g2[p] = gg; NB.pt2[p] = pt; NB.r2[p] = r;
                            NB.rab2[3 * p] = rab[0]; NB.rab2[3 * p + 1] = rab[1]; NB.rab2[3 * p + 2] = rab[2];
                        }
                        if (in3) { const int64_t p = o3 + c3 + __popc(b3 & lt); NB.g3[p] = gg; NB.r3[p] = r; }
                        if (in4) { const int64_t p = o4 + c4 + __popc(b4 & lt); NB.g4[p] = gg; NB.r4[p] = r; }
                    }
                    c2 += __popc(b2); c3 += __popc(b3); c4 += __popc(b4);
                }
            }
        }
    }
    if (!fill && lane == 0) { NB.cnt2[atom] = c2; NB.cnt3[atom] = c3; NB.cnt4[atom] = c4; }
}

// ---------------------------------------------------------------- clusters
__device__ __forceinline__ float dist32(const float4* c, int64_t a, int64_t b) {
    float4 x = c[a], y = c[b];
    float dx = y.x - x.x, dy = y.y - x.y, dz = y.z - x.z;
    return sqrtf(dx * dx + dy * dy + dz * dz);
}

// r(a,b) < smax decided exactly; FP32 settles all but the near-boundary cases.
__device__ __forceinline__ bool within(const FramesDev& F, const BoxDev& B, int64_t gbase, int a, int b,
                                       double smax, float r32) {
    if (r32 < (float)smax - MARGIN) return true;
    if (r32 > (float)smax + MARGIN) return false;
    double rab[3];
    double r = dist_exact(B.h, F.scaled + 3 * (gbase + a), F.scaled + 3 * (gbase + b), rab);
    return r < smax;
}

template <int NB_>
__global__ void k_clusters(ModelDev M, FramesDev F, NeighDev NB, ClusterSet CS, int fill, int parts) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int warp = gw / parts, part = gw - warp * parts;
    if (warp >= NB.n_real) return;
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (F.atom_ofs[mid] <= warp) lo = mid; else hi = mid - 1;
    }
    const int f = lo;
    const int N = F.natoms[f];
    const int i = warp - (int)F.atom_ofs[f];
    const int64_t gbase = F.ghost_ofs[f];
    const BoxDev& B = F.box[f];
    const int* typ = F.type + F.atom_ofs[f];
    const float4* c32 = reinterpret_cast<const float4*>(F.cart32);
    const int* lg = NB_ == 3 ? NB.g3 + NB.ofs3[warp] : NB.g4 + NB.ofs4[warp];
    const double* lr = NB_ == 3 ? NB.r3 + NB.ofs3[warp] : NB.r4 + NB.ofs4[warp];
    const int n = NB_ == 3 ? NB.cnt3[warp] : NB.cnt4[warp];
    const int* imap = NB_ == 3 ? M.int_map3 : M.int_map4;
    const int8_t* pidx = NB_ == 3 ? M.pidx3 : M.pidx4;
    const ClusterTypeDev* types = NB_ == 3 ? M.types3 : M.types4;
    const bool ordered = !B.small;
    const int ti = typ[i];
    int64_t out = fill ? CS.ofs[warp] : 0;
    if (fill)
        for (int q = 0; q < part; ++q) out += CS.pcnt[(int64_t)warp * parts + q];
    int count = 0;
    const int64_t total = NB_ == 3 ? (int64_t)n * n : (int64_t)n * n * n;
    const int64_t nbat = (total + 31) / 32;
    const int64_t b0 = nbat * part / parts * 32, b1 = min(total, nbat * (part + 1) / parts * 32);
    for (int64_t base = b0; base < b1; base += 32) {
        const int64_t t = base + lane;
        bool ok = false;
        int j = -1, k = -1, l = -1, T = -1;
        if (t < total) {
            int a, b, c = 0;
            if (NB_ == 3) { a = (int)(t / n); b = (int)(t % n); }
            else { a = (int)(t / ((int64_t)n * n)); b = (int)((t / n) % n); c = (int)(t % n); }
            j = lg[a]; k = lg[b];
            ok = (j != k) && !(ordered && (j % N) > (k % N));
            if (ok && NB_ == 4) {
                l = lg[c];
                ok = (j != l) && (k != l) && !(ordered && (k % N) > (l % N));
            }
            if (ok) {
                int id = (ti + 1) + 10 * (typ[j % N] + 1) + 100 * (typ[k % N] + 1) +
                         (NB_ == 4 ? 1000 * (typ[l % N] + 1) : 0);
                T = imap[id];
                ok = T >= 0;
                if (ok) {
                    const ClusterTypeDev& CT = types[T];
                    const int8_t* pm = pidx + id * (NB_ == 3 ? 3 : 6);
                    if (NB_ == 3) {
                        const double sk = NB.skin;
                        ok = lr[a] < CT.smax[pm[0]] + sk && lr[b] < CT.smax[pm[1]] + sk &&
                             within(F, B, gbase, j, k, CT.smax[pm[2]] + sk, dist32(c32, gbase + j, gbase + k));
                    } else {
                        const double sk = NB.skin;
                        ok = lr[a] < CT.smax[pm[0]] + sk && lr[b] < CT.smax[pm[1]] + sk && lr[c] < CT.smax[pm[2]] + sk &&
                             within(F, B, gbase, j, k, CT.smax[pm[3]] + sk, dist32(c32, gbase + j, gbase + k)) &&
                             within(F, B, gbase, j, l, CT.smax[pm[4]] + sk, dist32(c32, gbase + j, gbase + l)) &&
                             within(F, B, gbase, k, l, CT.smax[pm[5]] + sk, dist32(c32, gbase + k, gbase + l));
                    }
                }
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, ok);
        if (fill && ok) {
            int64_t p = out + count + __popc(bal & ((1u << lane) - 1u));
            CS.m[p] = make_int4(i, j, k, l);
            CS.type[p] = T;
        }
        count += __popc(bal);
    }
    if (!fill && lane == 0) {
        if (parts == 1) {
            CS.cnt[warp] = count;
        } else {
            CS.pcnt[(int64_t)warp * parts + part] = count;
            atomicAdd(CS.cnt + warp, count);
        }
    }
}

// Quadruplets in two stages (same accepted set as k_clusters<4>, different but fixed
// order): the lanes first test (j, k) pairs -- distinct, parent-ordered, r_jk under
// the largest 4-body cut-off -- and the surviving pairs of each chunk of 32 are then
// crossed with every l, flattened over the lanes, with the full per-slot tests.
__global__ void k_quads(ModelDev M, FramesDev F, NeighDev NB, ClusterSet CS, int fill, int parts) {
    __shared__ int2 sPair[8][32];
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int wib = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int warp = gw / parts, part = gw - warp * parts;
    if (warp >= NB.n_real) return;
    int lo = 0, hi = F.nframes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (F.atom_ofs[mid] <= warp) lo = mid; else hi = mid - 1;
    }
    const int f = lo;
    const int N = F.natoms[f];
    const int i = warp - (int)F.atom_ofs[f];
    const int64_t gbase = F.ghost_ofs[f];
    const BoxDev& B = F.box[f];
    const int* typ = F.type + F.atom_ofs[f];
    const float4* c32 = reinterpret_cast<const float4*>(F.cart32);
    const int* lg = NB.g4 + NB.ofs4[warp];
    const double* lr = NB.r4 + NB.ofs4[warp];
    const int n = NB.cnt4[warp];
    const bool ordered = !B.small;
    const int ti = typ[i];
    const float cut = (float)(M.maxcut4 + NB.skin) + MARGIN;
    int64_t out = fill ? CS.ofs[warp] : 0;
    if (fill)
        for (int q = 0; q < part; ++q) out += CS.pcnt[(int64_t)warp * parts + q];
    int count = 0;
    const int npairs = n * n;
    const unsigned lt = (1u << lane) - 1u;
    const int nbat = (npairs + 31) / 32;
    const int pb0 = nbat * part / parts * 32, pb1 = min(npairs, nbat * (part + 1) / parts * 32);
    for (int pb = pb0; pb < pb1; pb += 32) {
        const int p = pb + lane;
        bool pv = false;
        int a = 0, b = 0;
        if (p < npairs) {
            a = p / n; b = p - a * n;
            const int j = lg[a], k = lg[b];
            pv = (j != k) && !(ordered && (j % N) > (k % N)) && dist32(c32, gbase + j, gbase + k) < cut;
        }
        const unsigned pbal = __ballot_sync(0xffffffffu, pv);
        if (pv) sPair[wib][__popc(pbal & lt)] = make_int2(a, b);
        __syncwarp();
        const int work = __popc(pbal) * n;
        for (int tb = 0; tb < work; tb += 32) {
            const int t = tb + lane;
            bool ok = false;
            int j = -1, k = -1, l = -1, T = -1;
            if (t < work) {
                const int pi = t / n, c = t - pi * n;
                const int2 ab = sPair[wib][pi];
                j = lg[ab.x]; k = lg[ab.y]; l = lg[c];
                ok = (j != l) && (k != l) && !(ordered && (k % N) > (l % N));
                if (ok) {
                    const int id = (ti + 1) + 10 * (typ[j % N] + 1) + 100 * (typ[k % N] + 1) + 1000 * (typ[l % N] + 1);
                    T = M.int_map4[id];
                    ok = T >= 0;
                    if (ok) {
                        const ClusterTypeDev& CT = M.types4[T];
                        const int8_t* pm = M.pidx4 + id * 6;
                        const double sk = NB.skin;
                        ok = lr[ab.x] < CT.smax[pm[0]] + sk && lr[ab.y] < CT.smax[pm[1]] + sk &&
                             lr[c] < CT.smax[pm[2]] + sk &&
                             within(F, B, gbase, j, k, CT.smax[pm[3]] + sk, dist32(c32, gbase + j, gbase + k)) &&
                             within(F, B, gbase, j, l, CT.smax[pm[4]] + sk, dist32(c32, gbase + j, gbase + l)) &&
                             within(F, B, gbase, k, l, CT.smax[pm[5]] + sk, dist32(c32, gbase + k, gbase + l));
                    }
                }
            }
            const unsigned bal = __ballot_sync(0xffffffffu, ok);
            if (fill && ok) {
                const int64_t q = out + count + __popc(bal & lt);
                CS.m[q] = make_int4(i, j, k, l);
                CS.type[q] = T;
            }
            count += __popc(bal);
        }
        __syncwarp();
    }
    if (!fill && lane == 0) {
        if (parts == 1) {
            CS.cnt[warp] = count;
        } else {
            CS.pcnt[(int64_t)warp * parts + part] = count;
            atomicAdd(CS.cnt + warp, count);
        }
    }
}

// ---------------------------------------------------------------- bucketing
// Stable counting sort of one frame's items by key, one CTA per frame.  The items
// are split into contiguous ranges, one per warp (as many warps as the per-warp key
// counts fit in shared memory); each warp counts the keys of its range, a scan turns
// the counts into a start for every (key, warp), and each warp then places its range
// in order, 32 items at a time, ranking equal keys with __match_any_sync.  Within a
// key the items keep their order, so the result does not depend on timing.
constexpr int BUCKET_THREADS = 512;
constexpr int BUCKET_MAX_KEYS = 8192;
constexpr int BUCKET_SMEM_INTS = 24576;   // per-warp key counts + key starts (96 KB)

__device__ __forceinline__ void bucket_item(const BucketSpec& S, int N, int64_t base, int64_t t, int& key, int& val) {
    if (S.kind == 0) {
        int64_t p = base + (t >> 1);
        int e = (int)(t & 1);
        key = e == 0 ? S.i2[p] : S.g2[p] % N;
        val = (int)t;
    } else if (S.kind == 1) {
        int64_t q = base + t / S.nb;
        int e = (int)(t % S.nb);
        int4 mm = S.m[q];
        int g = e == 0 ? mm.x : (e == 1 ? mm.y : (e == 2 ? mm.z : mm.w));
        key = g % N;
        val = (int)((t / S.nb) * 4 + e);
    } else {
        key = S.type[base + t];
        val = (int)t;
    }
}

__global__ void __launch_bounds__(BUCKET_THREADS) k_bucket(FramesDev F, BucketSpec S, Buckets out) {
    extern __shared__ int bsm[];
    __shared__ int part[BUCKET_THREADS];
    const int f = blockIdx.x;
    const int N = F.natoms[f];
    // pair items live in the neighbour CSR, which is indexed by global real atom
    const int64_t base = S.item_frame_ofs[f];
    const int64_t nunits = S.item_frame_ofs[f + 1] - base;
    const int mult = S.kind == 0 ? 2 : (S.kind == 1 ? S.nb : 1);
    const int64_t nitems = nunits * mult;
    const int64_t kbase = S.key_frame_ofs[f];
    const int K = (int)(S.key_frame_ofs[f + 1] - kbase - 1);
    const int64_t vbase = base * mult;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int W = max(1, min((int)(blockDim.x >> 5), (BUCKET_SMEM_INTS - K) / max(K, 1)));
    int* cntw = bsm;            // [W][K]: counts, then starts
    int* kst = bsm + W * K;     // [K]: totals, then starts
    for (int k = threadIdx.x; k < W * K; k += blockDim.x) cntw[k] = 0;
    __syncthreads();
    const int64_t chunk = (nitems + W - 1) / W;
    const int64_t r0 = min(nitems, (int64_t)warp * chunk), r1 = min(nitems, r0 + chunk);
    if (warp < W) {
        for (int64_t t = r0 + lane; t < r1; t += 32) {
            int key, val;
            bucket_item(S, N, base, t, key, val);
            atomicAdd(&cntw[warp * K + key], 1);
        }
    }
    __syncthreads();
    // per key: starts of each warp's share relative to the key, and the key's total
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        int run = 0;
        for (int w = 0; w < W; ++w) { const int v = cntw[w * K + k]; cntw[w * K + k] = run; run += v; }
        kst[k] = run;
    }
    __syncthreads();
    // exclusive scan of the key totals
    const int per = (K + blockDim.x - 1) / blockDim.x;
    const int k0 = threadIdx.x * per, k1 = min(K, k0 + per);
    int local = 0;
    for (int k = k0; k < k1; ++k) local += kst[k];
    part[threadIdx.x] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < (int)blockDim.x; ++w) { int v = part[w]; part[w] = run; run += v; }
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int k = k0; k < k1; ++k) { int v = kst[k]; kst[k] = run; out.key_ofs[kbase + k] = vbase + run; run += v; }
    if (threadIdx.x == 0) out.key_ofs[kbase + K] = vbase + nitems;
    __syncthreads();
    for (int k = threadIdx.x; k < W * K; k += blockDim.x) cntw[k] += kst[k % K];
    __syncthreads();
    if (warp < W) {
        int* cnt = cntw + warp * K;
        for (int64_t c0 = r0; c0 < r1; c0 += 32) {
            int64_t t = c0 + lane;
            bool act = t < r1;
            int key = -1 - lane, val = 0;
            if (act) bucket_item(S, N, base, t, key, val);
            unsigned peers = __match_any_sync(0xffffffffu, key);
            int leader = __ffs(peers) - 1;
            int rank = __popc(peers & ((1u << lane) - 1u));
            int start = 0;
            if (act && lane == leader) start = cnt[key];
            start = __shfl_sync(0xffffffffu, start, leader);
            if (act) out.val[vbase + start + rank] = val;
            __syncwarp();
            if (act && lane == leader) cnt[key] = start + __popc(peers);
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------- launchers
void launch_frame_setup(const FramesDev& F, int64_t n, cudaStream_t st) {
    if (n > 0) k_frame_setup<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(F, n);
}
void launch_neigh(const ModelDev& M, const FramesDev& F, const NeighDev& NB, int fill, cudaStream_t st) {
    // enough atoms to fill the GPU with one warp each: one warp per atom
    if (NB.n_real <= 0) return;
    if (NB.n_real >= 32768)
        k_neigh<<<(unsigned)((NB.n_real + NEIGH_WARPS - 1) / NEIGH_WARPS), 32 * NEIGH_WARPS, 0, st>>>(M, F, NB, fill, 1);
    else
        k_neigh<<<(unsigned)NB.n_real, 32 * NEIGH_WARPS, 0, st>>>(M, F, NB, fill, NEIGH_WARPS);
}
void launch_bins(const FramesDev& F, int64_t n, const Bins& B, cudaStream_t st) {
    if (n <= 0) return;
    cudaMemsetAsync(B.count, 0, sizeof(int) * B.nbins, st);
    k_bin_count<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(F, n, B);
    launch_scan_counts(B.count, (int)B.nbins, B.start, st);
    cudaMemsetAsync(B.count, 0, sizeof(int) * B.nbins, st);
    k_bin_fill<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(F, n, B);
}

void launch_neigh_binned(const ModelDev& M, const FramesDev& F, const NeighDev& NB, const Bins& B, int fill,
                         cudaStream_t st) {
    if (NB.n_real > 0) k_neigh_binned<<<(unsigned)((NB.n_real + 7) / 8), 256, 0, st>>>(M, F, NB, B, fill);
}

int cluster_parts(int n_real) {
    return n_real >= 32768 ? 1 : n_real >= 16384 ? 2 : n_real >= 8192 ? 4 : 8;
}

void launch_clusters(int nbody, const ModelDev& M, const FramesDev& F, const NeighDev& NB, const ClusterSet& CS,
                     int fill, cudaStream_t st) {
    if (NB.n_real <= 0) return;
    const int parts = CS.pcnt ? cluster_parts(NB.n_real) : 1;
    if (parts > 1 && !fill) cudaMemsetAsync(CS.cnt, 0, sizeof(int) * NB.n_real, st);
    const unsigned g = (unsigned)(((int64_t)NB.n_real * parts + 7) / 8);
    if (nbody == 3) k_clusters<3><<<g, 256, 0, st>>>(M, F, NB, CS, fill, parts);
    else k_quads<<<g, 256, 0, st>>>(M, F, NB, CS, fill, parts);
}
void launch_bucket(int nframes, const FramesDev& F, const BucketSpec& S, const Buckets& out, cudaStream_t st) {
    if (nframes <= 0) return;
    const int smem = BUCKET_SMEM_INTS * (int)sizeof(int);
    cudaFuncSetAttribute(k_bucket, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_bucket<<<nframes, BUCKET_THREADS, smem, st>>>(F, S, out);
}

}  // namespace cgd
