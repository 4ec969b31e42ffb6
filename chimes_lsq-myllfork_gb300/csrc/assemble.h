// Launch configuration and shared-memory layout of the assembly kernels.
#pragma once
#include "kernels.h"

namespace cgd {

constexpr int MB_THREADS = 512;     // threads of the many-body kernels
constexpr int MB_CB = 16;           // clusters staged per shared-memory batch
// clusters per batch of the force kernel: twice as many in the FP32 form, whose
// tables take half the shared memory (half the batch barriers per owner atom)
__host__ __device__ constexpr int mb_force_cb(int rsize) { return rsize == 4 ? 32 : 16; }
constexpr int MB_MAX_ENT = 1024;    // owner incidences handled per pass
constexpr int VIR_PPT = 4;          // powers per thread in the stress/energy kernel
constexpr int VIR_CLUSTERS = 512;   // clusters per CTA in the stress/energy kernel
constexpr int F2_THREADS = 128;     // 2-body kernels

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

struct MbForceSmem {
    size_t ent, key, ord, cnt, q, pi, sg, gh, w, tab, total;
};
__host__ __device__ inline MbForceSmem mb_force_smem(int nbody, int ord, int nkeys, int max_allowed, int rsize) {
    const int np = nbody == 3 ? 3 : 6, ni = nbody - 1, no = np - ni;
    int sizeI = 1, sizeO = 1;
    for (int k = 0; k < ni; ++k) sizeI *= ord;
    for (int k = 0; k < no; ++k) sizeO *= ord;
    const size_t per = 3 * (size_t)sizeI + sizeO;
    MbForceSmem s;
    s.ent = 0;
    s.key = align16(s.ent + MB_MAX_ENT * sizeof(int));
    s.ord = align16(s.key + MB_MAX_ENT * sizeof(int));
    s.cnt = align16(s.ord + MB_MAX_ENT * sizeof(int));
    s.q = align16(s.cnt + (nkeys + 1) * sizeof(int));
    const int cb = mb_force_cb(rsize);
    s.pi = align16(s.q + cb * sizeof(int));
    s.sg = align16(s.pi + cb * sizeof(int));
    s.gh = align16(s.sg + cb * 6 * sizeof(int));
    s.w = align16(s.gh + (size_t)cb * np * 2 * ord * rsize);
    s.tab = align16(s.w + (size_t)cb * np * 3 * ord * rsize);
    size_t tab = (size_t)cb * per;
    if ((size_t)max_allowed * 3 > tab) tab = (size_t)max_allowed * 3;
    s.total = align16(s.tab + tab * rsize);
    return s;
}

// Range form of the force kernel (k_force_rg): at most rg_max_threads threads, two CTAs
// per SM (384 in FP64, where 80 registers a thread keep the FMA loop out of local
// memory; 512 in FP32, whose shorter latency-bound loop gains from the extra warps).
// Shared memory: the incidence sort, then per chunk of mb_force_cb clusters (of every
// owner role) the slot bases, the owner-weighted derivatives and the M / Q tables,
// and one partial column sum (3 values) per thread.
__host__ __device__ constexpr int rg_max_threads(int rsize) { return rsize == 8 ? 384 : 512; }
struct MbRangeSmem {
    size_t ent, key, ord, cnt, q, m, role, sg, gh, w, tab, part, total;
};
__host__ __device__ inline MbRangeSmem mb_range_smem(int nbody, int ord, int nkeys, int nt, int rsize) {
    const int np = nbody == 3 ? 3 : 6, ni = nbody - 1, no = np - ni;
    int sizeI = 1, sizeO = 1;
    for (int k = 0; k < ni; ++k) sizeI *= ord;
    for (int k = 0; k < no; ++k) sizeO *= ord;
    const size_t per = 3 * (size_t)sizeI + sizeO;
    const int cb = mb_force_cb(rsize);
    MbRangeSmem s;
    s.ent = 0;
    s.key = align16(s.ent + MB_MAX_ENT * sizeof(int));
    s.ord = align16(s.key + MB_MAX_ENT * sizeof(int));
    s.cnt = align16(s.ord + MB_MAX_ENT * sizeof(int));
    s.q = align16(s.cnt + (nkeys + 1) * sizeof(int));
    s.m = align16(s.q + cb * sizeof(int));
    s.role = align16(s.m + cb * sizeof(int));
    s.sg = align16(s.role + cb * sizeof(int));
    s.gh = align16(s.sg + cb * 6 * sizeof(int));
    s.w = align16(s.gh + (size_t)cb * np * 2 * ord * rsize);
    s.tab = align16(s.w + (size_t)cb * np * 3 * ord * rsize);
    s.part = align16(s.tab + (size_t)cb * per * rsize);
    s.total = align16(s.part + (size_t)nt * 3 * rsize);
    return s;
}

struct MbVirSmem {
    size_t q, gh, v, tab, total;
};
__host__ __device__ inline MbVirSmem mb_vir_smem(int nbody, int ord, int pchunk, int rsize) {
    const int np = nbody == 3 ? 3 : 6, n1 = nbody - 1, n2 = np - n1;
    int s1 = 1, s2 = 1;
    for (int k = 0; k < n1; ++k) s1 *= ord;
    for (int k = 0; k < n2; ++k) s2 *= ord;
    const size_t per = 7 * (size_t)s1 + 7 * (size_t)s2;
    MbVirSmem s;
    s.q = 0;
    s.gh = align16(MB_CB * sizeof(int));
    s.v = align16(s.gh + (size_t)MB_CB * np * 2 * ord * rsize);
    s.tab = align16(s.v + (size_t)MB_CB * np * 6 * rsize);
    size_t tab = (size_t)MB_CB * per;
    if ((size_t)pchunk * 7 > tab) tab = (size_t)pchunk * 7;
    s.total = align16(s.tab + tab * rsize);
    return s;
}

// Energy (comp 0) and stress (comps 1..6 = xx yy zz xy xz yz) rows of one column,
// in the reference's row order (src/A_Matrix.C:309-553).
template <typename R>
__device__ __forceinline__ void write_virial_rows(const FramesDev& F, int f, int64_t col, const R* s, double inv_vol,
                                                  R* A, int64_t lda) {
    const int N = F.natoms[f];
    const int sr = F.stress_rows[f], er = F.energy_rows[f];
    int64_t row = F.row_ofs[f] + 3 * (int64_t)N;
    if (sr == 3) {
        A[(row + 0) * lda + col] = R(s[1] * inv_vol);
        A[(row + 1) * lda + col] = R(s[2] * inv_vol);
        A[(row + 2) * lda + col] = R(s[3] * inv_vol);
    } else if (sr == 9) {
        const int map9[9] = {1, 4, 5, 4, 2, 6, 5, 6, 3};
        for (int k = 0; k < 9; ++k) A[(row + k) * lda + col] = R(s[map9[k]] * inv_vol);
    }
    row += sr;
    for (int k = 0; k < er; ++k) A[(row + k) * lda + col] = s[0];
}

// Host launchers (kernels are defined in assemble.cu).  prec: 0 FP64, 1 FP32.
void launch_force2(int prec, int nreal, const ModelDev& M, const FramesDev& F, const NeighDev& NB,
                   const Buckets& inc, const int64_t* key_frame_ofs, void* A, int64_t lda, cudaStream_t st);
// 2-body stress/energy rows in two launches: per-(frame, slice) partials into part
// (nframes * nslice * 7 * 2-body columns values in the form's type), then the rows.
int virial2_slices(int nframes, int64_t npairs, int sms);
void launch_virial2(int prec, int nframes, int nslice, const ModelDev& M, const FramesDev& F, const NeighDev& NB,
                    void* part, void* A, int64_t lda, cudaStream_t st);
// Slot bases of every cluster, once per cluster: [cluster][slot][2 ord + 4] values in
// the form's type (g, h, r, r_ab), read by the force and stress/energy kernels.
size_t cluster_basis_count(int nbody, int ord, int64_t nclusters);
void launch_cluster_basis(int nbody, int prec, int64_t nclusters, const ModelDev& M, const FramesDev& F,
                          const ClusterSet& CS, void* basis, cudaStream_t st);
// pre: the cluster bases above, or nullptr to evaluate them in the kernel.  nt4:
// threads per CTA of the 4-body kernel when it needs more than two powers per thread
// (MB_THREADS or 2 * MB_THREADS).
void launch_force_mb(int nbody, int prec, int ppt, int nreal, size_t smem, const ModelDev& M, const FramesDev& F,
                     const ClusterSet& CS, const Buckets& inc, const int64_t* key_frame_ofs, const void* pre,
                     void* A, int64_t lda, cudaStream_t st, int nt4 = MB_THREADS);
// The same rows by the range form (k_force_rg) on nt threads per CTA;
// smem = mb_range_smem(..., nt, ...).total.
void launch_force_rg(int nbody, int prec, int nreal, int nt, size_t smem, const ModelDev& M, const FramesDev& F,
                     const ClusterSet& CS, const Buckets& inc, const int64_t* key_frame_ofs, const void* pre,
                     void* A, int64_t lda, cudaStream_t st);
// Threads per CTA of k_force_rg.  FP64: the multiple of 32 in [max / 2, max] whose
// ranges of ceil(n / threads) powers leave the fewest idle lanes (which still occupy
// the FP64 pipe) over the cluster types' allowed-power counts; FP32: the maximum.
int rg_threads(const int* n_allowed, int ntypes, int rsize);
// Stress/energy rows: nchunks_max cluster chunks of VIR_CLUSTERS per (frame, type);
// part holds nframes*ntypes*nchunks_max*7*ntrue_max partial sums (R).
// ppt: powers per thread, 1 when every cluster type has at most MB_THREADS allowed
// powers (fewer registers, more CTAs per SM), else VIR_PPT.
void launch_virial_mb(int nbody, int prec, int ppt, int nframes, int ntypes, int nzchunk, int nchunks_max,
                      int ntrue_max, size_t smem, const ModelDev& M, const FramesDev& F, const ClusterSet& CS,
                      const Buckets& byt, const int64_t* key_frame_ofs, int ncomp, const void* pre, void* part,
                      void* A, int64_t lda, cudaStream_t st);
void launch_max_bucket(const int64_t* key_ofs, const int64_t* key_frame_ofs, int nframes, int ntypes, int* out,
                       cudaStream_t st);
void launch_energy_cols(int prec, int nframes, const ModelDev& M, const FramesDev& F, void* A, int64_t lda,
                        cudaStream_t st);
// FITCOUL charge columns of the force rows (ewald.cu): real space, structure
// factors, k space; S holds ewald_scratch_bytes(nframes, natmtyp).
size_t ewald_scratch_bytes(int nframes, int natmtyp);
void launch_ewald(int prec, int nframes, int nreal, const ModelDev& M, const FramesDev& F, void* S, void* A,
                  int64_t lda, cudaStream_t st);

}  // namespace cgd
