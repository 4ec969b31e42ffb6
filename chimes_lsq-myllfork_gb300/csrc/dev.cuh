// Device-side data layout shared by the design-matrix and MD-force kernels.
//
// Everything here is plain structs of device pointers; the host fills them in
// session.cu.  Geometry decisions (which pairs / triplets / quadruplets exist)
// use explicitly rounded FP64 intrinsics so that they repeat the reference's
// rounding sequence exactly (BOX::GET_DISTANCE src/ClassDefs.C:2321-2358,
// get_dist src/functions.h:655-667); the basis arithmetic may contract.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace cgd {

constexpr int MAXB = 4;        // maximum bodiedness
constexpr int MAXS = 6;        // slots (pairs) of a 4-body cluster
constexpr int MAXORD = 24;     // largest Chebyshev order supported on the device
constexpr int MAXCHUNK = 16;   // power chunks of one cluster type in the stress/energy kernel

// ---------------------------------------------------------------- model tables
struct PairDev {               // one 2-body pair type
    double smin, smax, lambda, xavg, xdiff;
    int col;                   // first A column of its 2-body block, -1 when HIERARC excludes it
};

struct ClusterTypeDev {        // one triplet / quadruplet type
    int n_allowed, n_true, col_base;
    int pow_offset;            // into ModelDev::powN (n_allowed * nslots bytes)
    int grp_offset;            // into ModelDev::grpN (n_true + 1 ints)
    int vir_nchunk;            // power chunks (group aligned) of the stress/energy kernel
    int vir_chunk[MAXCHUNK + 1];
    double smax[MAXS], smin[MAXS], xavg[MAXS], xdiff[MAXS], lambda[MAXS];
};

struct ModelDev {
    int natmtyp, npairs;
    int order2, order3, order4;          // Chebyshev orders (2B columns use T_1..T_order2)
    int trans, fix, fcut;                // ChebTrans / ChebFix / FcutKind
    double smooth, deriv_const, fcut_offset;
    double maxcut2, maxcut3, maxcut4;    // exact list cut-offs (no padding)
    int ntypes3, ntypes4;
    int n2b, tot_short, tot_all;         // column counts
    int col3, col4;                      // first 3B / 4B column
    int fit_ener_cols;                   // atom types scanned for energy-offset columns (0 or natmtyp)
    int ener_col[10];                    // energy-offset column of each type after tot_short + ncoul; -1 excluded
    int ncoul;                           // FITCOUL charge columns (one per pair type), after tot_short
    const int* int_pair_map;             // natmtyp^2
    const PairDev* pairs;
    const int* int_map3;                 // 1000 entries
    const int8_t* pidx3;                 // 1000 * 3   actual edge -> canonical slot
    const int8_t* rev3;                  // 1000 * 3   actual member -> canonical position
    const ClusterTypeDev* types3;
    const uint8_t* pow3;
    const int* grp3;
    const int* int_map4;                 // 10000 entries
    const int8_t* pidx4;                 // 10000 * 6
    const int8_t* rev4;                  // 10000 * 4
    const ClusterTypeDev* types4;
    const uint8_t* pow4;
    const int* grp4;
    // Per allowed power (indexed pow_offset / nslots + p): for each canonical role pi
    // of the owner, the power's entries in a cluster's force table (see k_force_rg):
    // low 16 bits the M_x index, high 16 bits the Q index.  And the column of the
    // power within its type (PARAM_INDICES).
    const uint4* offs3;
    const int* tcol3;
    const uint4* offs4;
    const int* tcol4;
};

// Canonical slots incident to the member at canonical position pi (nb - 1 of them,
// k-th returned by role_slot_in) and the other slots (role_slot_out).  Edges of a
// triplet: 0 = (0,1), 1 = (0,2), 2 = (1,2); of a quadruplet: 0 = (0,1), 1 = (0,2),
// 2 = (0,3), 3 = (1,2), 4 = (1,3), 5 = (2,3).  Packed 4 bits per entry:
//   3-body in  {0,1} {0,2} {1,2}                out {2} {1} {0}
//   4-body in  {0,1,2} {0,3,4} {1,3,5} {2,4,5}  out {3,4,5} {1,2,5} {0,2,4} {0,1,3}
__host__ __device__ constexpr int role_slot_in(int nb, int pi, int k) {
    return nb == 3 ? (int)((0x212010ull >> (4 * (2 * pi + k))) & 15) : (int)((0x542531430210ull >> (4 * (3 * pi + k))) & 15);
}
__host__ __device__ constexpr int role_slot_out(int nb, int pi, int k) {
    return nb == 3 ? (int)((0x012ull >> (4 * pi)) & 15) : (int)((0x310420521543ull >> (4 * (3 * pi + k))) & 15);
}

// ---------------------------------------------------------------- frame batch
struct BoxDev {
    double h[9], inv[9];
    double lx, ly, lz, vol;
    int is_ortho, small;                 // small = unordered neighbour convention
    double perm2, perm3, perm4;          // PERM_SCALE[n]
    double ew_alpha, ew_rc;              // Ewald splitting and real-space cut-off (FITCOUL)
    int ew_kmax;                         // Ewald integer k cut-off
};

struct FramesDev {
    int nframes, nlayers, nimg;          // nimg = (2L+1)^3
    const int* natoms;                   // [nframes]
    const int64_t* atom_ofs;             // [nframes+1]
    const int64_t* ghost_ofs;            // [nframes+1] (nimg * natoms prefix)
    const int64_t* row_ofs;              // [nframes+1] A-matrix row offsets
    const int* stress_rows;              // [nframes] 0, 3 or 9
    const int* energy_rows;              // [nframes] 0 or 3
    const BoxDev* box;                   // [nframes]
    const int* type;                     // [atoms]
    const double* xyz;                   // [atoms*3]
    // derived by k_frame_setup
    double* scaled;                      // [ghosts*3] H^-1 x of every real and ghost atom
    float* cart32;                       // [ghosts*4] FP32 Cartesian copy for the pre-filter
    // MD list reuse: the lattice shift that wraps each atom, computed when the lists
    // are built (shift_mode 1) and reused until the next build (shift_mode 2), so a
    // ghost index names the same image while atoms move.  null / 0: wrap each call.
    int* shift;                          // [atoms*3]
    int shift_mode;
};

// ---------------------------------------------------------------- exact FP64
#ifdef __CUDACC__
__device__ __forceinline__ double mulrn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double addrn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double subrn(double a, double b) { return __dsub_rn(a, b); }

// ((m0*x + m1*y) + m2*z) with one rounding per operation, as the reference's
// x86-64 build evaluates it (no fused multiply-add).
__device__ __forceinline__ double dot3rn(double m0, double m1, double m2, double x, double y, double z) {
    return addrn(addrn(mulrn(m0, x), mulrn(m1, y)), mulrn(m2, z));
}

// Distance a2 - a1 from pre-scaled coordinates; returns |r| and the vector.
__device__ __forceinline__ double dist_exact(const double* __restrict__ h, const double* s1,
                                             const double* s2, double* rab) {
    double tx = subrn(s2[0], s1[0]), ty = subrn(s2[1], s1[1]), tz = subrn(s2[2], s1[2]);
    rab[0] = dot3rn(h[0], h[1], h[2], tx, ty, tz);
    rab[1] = dot3rn(h[3], h[4], h[5], tx, ty, tz);
    rab[2] = dot3rn(h[6], h[7], h[8], tx, ty, tz);
    return __dsqrt_rn(addrn(addrn(mulrn(rab[0], rab[0]), mulrn(rab[1], rab[1])), mulrn(rab[2], rab[2])));
}

// Layer k (0-based over the (2L+1)^3-1 non-zero layers in n1,n2,n3 order).
__device__ __forceinline__ void layer_index(int k, int L, int& n1, int& n2, int& n3) {
    int side = 2 * L + 1;
    int center = (side * side * side) / 2;
    int lin = k < center ? k : k + 1;
    n1 = lin / (side * side) - L;
    n2 = (lin / side) % side - L;
    n3 = lin % side - L;
}
#endif  // __CUDACC__

}  // namespace cgd
