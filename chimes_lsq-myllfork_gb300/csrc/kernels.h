// Device work lists produced by the enumeration kernels and consumed by the
// assembly kernels, plus the kernel entry points.
#pragma once
#include "dev.cuh"

namespace cgd {

struct NeighDev {
    int n_real;                                   // real atoms in the batch (one list each)
    int* cnt2; int* cnt3; int* cnt4;              // [n_real]
    int64_t* ofs2; int64_t* ofs3; int64_t* ofs4;  // [n_real + 1] exclusive prefix
    // 2-body pairs accepted by s_min < r < s_max (src/Cheby.C:772)
    int* i2; int* g2; int* pt2; double* r2; double* rab2;
    // 3-body / 4-body candidate lists: r < maximum cluster cut-off
    int* g3; double* r3;
    int* g4; double* r4;
    // 0: the fit's 2-body filter s_min < r < s_max; 1: the MD force's r < s_max
    // (Cheby::Force_all src/Cheby.C:1834 also evaluates r <= s_min, smoothed);
    // 2: MD lists reused over steps (pair distances recomputed, r < s_max tested)
    int md;
    // MD list reuse: every cut-off of the enumeration widened by this skin (0: exact)
    double skin;
};

struct ClusterSet {                               // triplets or quadruplets of a batch
    int* cnt;                                     // [n_real] clusters centred on each real atom
    int64_t* ofs;                                 // [n_real + 1]
    int4* m;                                      // members (frame-local ghost indices), .w = -1 for 3B
    int* type;                                    // cluster type index
    int* pcnt = nullptr;                          // [n_real * cluster_parts(n_real)] when that is > 1
};

// Warps that share one centre atom's enumeration (1, 2, 4 or 8): small batches
// split each atom's candidate range so the GPU has enough warps; the clusters
// keep the order of a single warp's walk.
int cluster_parts(int n_real);

// Stable per-frame bucketing (owner incidences and per-type lists).
struct Buckets {
    int64_t* key_ofs;                             // [sum_f K_f + nframes] global start of each (frame,key)
    int* val;                                     // permuted item values
};

// Per-frame item ranges for a bucketing pass.
struct BucketSpec {
    int kind;                                     // 0: 2B pair ends, 1: cluster members, 2: cluster types
    int nb;                                       // members per cluster (kind 1)
    const int64_t* item_frame_ofs;                // [nframes+1] (in pairs / clusters)
    const int64_t* key_frame_ofs;                 // [nframes+1] (in keys, incl. one sentinel per frame)
    const int* i2;                                // kind 0
    const int* g2;                                // kind 0
    const int4* m;                                // kind 1
    const int* type;                              // kind 2
};

// Cell grid of one frame for the binned neighbour search: bins in fractional
// coordinates over the ghost-extended cell, each at least the search radius wide
// along its reciprocal direction, so neighbours lie in adjacent bins.
struct BinGrid {
    int nb[3];
    int64_t ofs;                                  // first bin of the frame in the batch
};
struct Bins {
    const BinGrid* grid;                          // [nframes]
    int64_t nbins;
    int* count;                                   // [nbins] then fill cursors
    int64_t* start;                               // [nbins + 1]
    int* atoms;                                   // [ghosts] frame-local ghost indices, grouped by bin
};

// Host launchers (kernels are defined in geom.cu).
void launch_frame_setup(const FramesDev& F, int64_t total_ghosts, cudaStream_t st);
void launch_neigh(const ModelDev& M, const FramesDev& F, const NeighDev& NB, int fill, cudaStream_t st);
void launch_clusters(int nbody, const ModelDev& M, const FramesDev& F, const NeighDev& NB, const ClusterSet& CS,
                     int fill, cudaStream_t st);
void launch_bucket(int nframes, const FramesDev& F, const BucketSpec& S, const Buckets& out, cudaStream_t st);
// Binned neighbour lists (MD list builds): bin every ghost, then the same count /
// fill passes as launch_neigh over the 27 bins around each real atom (list order
// follows the bins, not the ghost index).
void launch_bins(const FramesDev& F, int64_t total_ghosts, const Bins& B, cudaStream_t st);
void launch_neigh_binned(const ModelDev& M, const FramesDev& F, const NeighDev& NB, const Bins& B, int fill,
                         cudaStream_t st);
// Prefix sums and per-frame offsets (session.cu).
void launch_scan_counts(const int* cnt, int n, int64_t* ofs, cudaStream_t st);
void launch_gather_frame_ofs(const int64_t* ofs, const int64_t* atom_ofs, int nframes, int64_t* out, cudaStream_t st);
void launch_key_frame_ofs(const int64_t* atom_ofs, int nframes, int per_type, int64_t* out, cudaStream_t st);

}  // namespace cgd
