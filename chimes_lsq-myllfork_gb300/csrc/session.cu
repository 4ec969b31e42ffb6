// Host orchestration of the design-matrix path (see session.h).
#include "session.h"

#include <sys/mman.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <numeric>

#include "../../include/chimes_gb300.h"
#include "dense64.h"
#include "gram.h"
#include "assemble.h"
#include "kernels.h"
#include "scratch.h"

namespace cg {

static const double GPA = 6.9476955;   // src/functions.h:45

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw Error(3, std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

template <typename T>
static T* dev_upload(std::vector<void*>& allocs, const T* src, size_t n) {
    T* p = nullptr;
    size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
    CK(cudaMalloc((void**)&p, bytes));
    allocs.push_back(p);
    if (n) CK(cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return p;
}

// ------------------------------------------------------------------ model tables
static void rev_index(const ClusterType& ct, const int* types, int n, int8_t* out) {
    std::vector<bool> used(n, false);   // greedy match of CLUSTER::map_indices_int src/Cluster.C:1813-1825
    for (int m = 0; m < n; ++m) {
        out[m] = -1;
        for (int q = 0; q < n; ++q)
            if (types[m] == ct.atom_indices[q] && !used[q]) { out[m] = (int8_t)q; used[q] = true; break; }
    }
}

static void upload_list(const Model& m, const ClusterList& cl, int nb, int ord, int col_base, int pchunk, DeviceModel& D,
                        const int** int_map, const int8_t** pidx, const int8_t** rev, const cgd::ClusterTypeDev** types,
                        const uint8_t** pows, const int** grps, const uint4** offs, const int** tcols, int& max_allowed) {
    const int np = nb == 3 ? 3 : 6;
    const int dim = nb == 3 ? 1000 : 10000;
    std::vector<int> imap(dim, -1);
    std::vector<int8_t> pi(dim * np, -1), rv(dim * nb, -1);
    for (int id = 0; id < dim && id < (int)cl.int_map.size(); ++id) {
        imap[id] = cl.int_map[id];
        if (imap[id] < 0) continue;
        for (int e = 0; e < np; ++e) pi[id * np + e] = (int8_t)cl.pair_indices[id][e];
        int t[4], x = id;
        for (int k = 0; k < nb; ++k) { t[k] = x % 10 - 1; x /= 10; }
        rev_index(cl.vec[imap[id]], t, nb, &rv[id * nb]);
    }
    std::vector<cgd::ClusterTypeDev> tv(cl.vec.size());
    std::vector<uint8_t> pw;
    std::vector<int> gp;
    std::vector<uint4> of;      // force-table entries of each power for each owner role
    std::vector<int> tc;        // column of each power within its type
    int sizeI = 1, sizeO = 1;
    for (int k = 0; k < nb - 1; ++k) sizeI *= ord;
    for (int k = 0; k < np - nb + 1; ++k) sizeO *= ord;
    if (3 * sizeI + sizeO > 65536) throw Error(2, "cluster order too large for the force-table offsets");
    int col = col_base;
    max_allowed = 0;
    for (size_t t = 0; t < cl.vec.size(); ++t) {
        const ClusterType& ct = cl.vec[t];
        cgd::ClusterTypeDev& d = tv[t];
        std::memset(&d, 0, sizeof(d));
        d.n_allowed = ct.excluded ? 0 : ct.n_allowed;
        d.n_true = ct.excluded ? 0 : ct.n_true;
        d.col_base = col;
        col += d.n_true;
        d.pow_offset = (int)pw.size();
        d.grp_offset = (int)gp.size();
        max_allowed = std::max(max_allowed, d.n_allowed);
        for (int p = 0; p < d.n_allowed; ++p)
            for (int s = 0; s < np; ++s) pw.push_back((uint8_t)ct.allowed_powers[p][s]);
        for (int p = 0; p < d.n_allowed; ++p) {
            uint32_t e[4] = {0, 0, 0, 0};
            for (int pi = 0; pi < nb; ++pi) {
                int ii = 0, oo = 0;
                for (int k = nb - 2; k >= 0; --k) ii = ii * ord + ct.allowed_powers[p][cgd::role_slot_in(nb, pi, k)];
                for (int k = np - nb; k >= 0; --k) oo = oo * ord + ct.allowed_powers[p][cgd::role_slot_out(nb, pi, k)];
                e[pi] = (uint32_t)ii | ((uint32_t)(3 * sizeI + oo) << 16);
            }
            of.push_back(make_uint4(e[0], e[1], e[2], e[3]));
            tc.push_back(ct.param_indices[p]);
        }
        // column groups: PARAM_INDICES is non-decreasing with contiguous groups
        int c = 0;
        for (int p = 0; p < d.n_allowed; ++p) {
            if (p > 0 && ct.param_indices[p] < ct.param_indices[p - 1])
                throw Error(2, "PARAM_INDICES not monotone; unsupported cluster layout");
            while (c <= ct.param_indices[p]) { gp.push_back(p); ++c; }
        }
        while (c <= d.n_true) { gp.push_back(d.n_allowed); ++c; }
        // group-aligned power chunks for the stress/energy kernel
        int nch = 0;
        d.vir_chunk[0] = 0;
        int start = 0;
        while (start < d.n_allowed) {
            int end = std::min(d.n_allowed, start + pchunk);
            if (end < d.n_allowed) {   // move back to a group start
                int gstart = end;
                while (gstart > start && ct.param_indices[gstart] == ct.param_indices[gstart - 1]) --gstart;
                if (gstart == start) throw Error(2, "power group larger than a chunk");
                end = gstart;
            }
            if (nch >= cgd::MAXCHUNK) throw Error(2, "too many power chunks for one cluster type");
            d.vir_chunk[++nch] = end;
            start = end;
        }
        d.vir_nchunk = nch;
        for (int s = 0; s < np; ++s) {
            d.smax[s] = ct.smax[s]; d.smin[s] = ct.smin[s]; d.xavg[s] = ct.xavg[s]; d.xdiff[s] = ct.xdiff[s];
            size_t j = 0;
            for (; j < m.pairs.size(); ++j) if (m.pairs[j].prpr == ct.pair_names[s]) break;
            d.lambda[s] = j < m.pairs.size() ? m.pairs[j].lambda : 0.0;
        }
    }
    *int_map = dev_upload(D.allocs, imap.data(), imap.size());
    *pidx = dev_upload(D.allocs, pi.data(), pi.size());
    *rev = dev_upload(D.allocs, rv.data(), rv.size());
    *types = dev_upload(D.allocs, tv.data(), tv.size());
    *pows = dev_upload(D.allocs, pw.data(), pw.size());
    *grps = dev_upload(D.allocs, gp.data(), gp.size());
    if (of.empty()) { of.push_back(make_uint4(0, 0, 0, 0)); tc.push_back(0); }
    *offs = dev_upload(D.allocs, of.data(), of.size());
    *tcols = dev_upload(D.allocs, tc.data(), tc.size());
}

DeviceModel::DeviceModel(const Model& m, int vir_pchunk) {
    const Controls& c = m.ctl;
    if (c.cheby_order > cgd::MAXORD || c.cheby3 > cgd::MAXORD || c.cheby4 > cgd::MAXORD)
        throw Error(2, "Chebyshev order above the device limit");
    if (c.use4 && c.cheby4 > 4) throw Error(2, "4-body order above 4 is not supported on the device");
    if (c.use3 && c.cheby3 > 16) throw Error(2, "3-body order above 16 is not supported on the device");
    cgd::ModelDev& d = dev;
    d.natmtyp = c.natmtyp;
    d.npairs = (int)m.pairs.size();
    d.order2 = c.cheby_order;
    d.order3 = c.use3 ? c.cheby3 : 0;
    d.order4 = c.use4 ? c.cheby4 : 0;
    d.trans = c.trans; d.fix = c.fix; d.fcut = c.fcut;
    d.smooth = c.smooth; d.deriv_const = m.deriv_const; d.fcut_offset = c.fcut_offset;
    d.maxcut2 = m.max_cutoff_2b; d.maxcut3 = m.max_cutoff_3b; d.maxcut4 = m.max_cutoff_4b;
    d.ntypes3 = c.use3 ? (int)m.trips.vec.size() : 0;
    d.ntypes4 = c.use4 ? (int)m.quads.vec.size() : 0;
    d.n2b = m.tot_snum; d.tot_short = m.tot_short; d.tot_all = m.tot_all;
    d.col3 = m.tot_snum; d.col4 = m.tot_snum + m.num3;
    d.fit_ener_cols = c.fit_ener ? c.natmtyp : 0;
    if (c.natmtyp > 10) throw Error(2, "more than 10 atom types");
    for (int t = 0; t < 10; ++t) d.ener_col[t] = t < c.natmtyp ? m.ener_col[t] : -1;
    d.ncoul = m.ncoul;
    d.int_pair_map = dev_upload(allocs, m.int_pair_map.data(), m.int_pair_map.size());
    std::vector<cgd::PairDev> pv;
    for (const auto& p : m.pairs) pv.push_back({p.smin, p.smax, p.lambda, p.xavg, p.xdiff, p.col});
    d.pairs = dev_upload(allocs, pv.data(), pv.size());
    if (c.use3)
        upload_list(m, m.trips, 3, c.cheby3, d.col3, vir_pchunk, *this, &d.int_map3, &d.pidx3, &d.rev3, &d.types3,
                    &d.pow3, &d.grp3, &d.offs3, &d.tcol3, max_allowed3);
    if (c.use4)
        upload_list(m, m.quads, 4, c.cheby4, d.col4, vir_pchunk, *this, &d.int_map4, &d.pidx4, &d.rev4, &d.types4,
                    &d.pow4, &d.grp4, &d.offs4, &d.tcol4, max_allowed4);
}

DeviceModel::~DeviceModel() {
    for (void* p : allocs) cudaFree(p);
}

// ------------------------------------------------------------------ frames
void set_small(cgd::BoxDev& bd, bool small) {
    bd.small = small ? 1 : 0;
    // PERM_SCALE src/ClassDefs.C:146-152
    bd.perm2 = small ? 0.5 : 1.0;
    bd.perm3 = small ? 0.5 / 3.0 : 1.0;
    bd.perm4 = small ? 0.5 / 3.0 / 4.0 : 1.0;
}

FrameBatch slice_batch(const FrameBatch& fb, int first, int count) {
    if (first < 0 || count < 0 || first + count > fb.nframes) throw Error(1, "frame range outside the batch");
    FrameBatch o;
    o.nframes = count;
    o.first_index = fb.first_index + first;
    o.nprocs = fb.nprocs;
    o.atom_ofs.push_back(0); o.ghost_ofs.push_back(0); o.row_ofs.push_back(0);
    const int64_t nimg = fb.natoms.empty() ? 1 : (fb.ghost_ofs[1] - fb.ghost_ofs[0]) / std::max(1, fb.natoms[0]);
    for (int k = first; k < first + count; ++k) {
        const int n = fb.natoms[k];
        o.natoms.push_back(n);
        o.stress_rows.push_back(fb.stress_rows[k]);
        o.energy_rows.push_back(fb.energy_rows[k]);
        o.box.push_back(fb.box[k]);
        o.small_self.push_back(fb.small_self[k]);
        o.file.push_back(k < (int)fb.file.size() ? fb.file[k] : 0);
        o.rank.push_back(k < (int)fb.rank.size() ? fb.rank[k] : 0);
        o.atom_ofs.push_back(o.atom_ofs.back() + n);
        o.ghost_ofs.push_back(o.ghost_ofs.back() + nimg * n);
        const int64_t rows = fb.row_ofs[k + 1] - fb.row_ofs[k];
        o.row_ofs.push_back(o.row_ofs.back() + rows);
        o.type.insert(o.type.end(), fb.type.begin() + fb.atom_ofs[k], fb.type.begin() + fb.atom_ofs[k + 1]);
        o.xyz.insert(o.xyz.end(), fb.xyz.begin() + 3 * fb.atom_ofs[k], fb.xyz.begin() + 3 * fb.atom_ofs[k + 1]);
        o.b.insert(o.b.end(), fb.b.begin() + fb.row_ofs[k], fb.b.begin() + fb.row_ofs[k + 1]);
    }
    o.nrows = o.row_ofs.back();
    o.natoms_total = o.atom_ofs.back();
    o.nghosts = o.ghost_ofs.back();
    return o;
}

void make_independent(FrameBatch& fb) {
    for (int k = 0; k < fb.nframes; ++k) set_small(fb.box[k], fb.small_self[k] != 0);
}

FrameBatch make_batch(const Model& m, const std::vector<Frame>& frames, int first_index, int nprocs) {
    FrameBatch fb;
    fb.nframes = (int)frames.size();
    fb.first_index = first_index;
    fb.nprocs = nprocs;
    const int L = m.ctl.nlayers;
    const int nimg = (2 * L + 1) * (2 * L + 1) * (2 * L + 1);
    fb.atom_ofs.push_back(0); fb.ghost_ofs.push_back(0); fb.row_ofs.push_back(0);
    bool small = false;
    for (int k = 0; k < fb.nframes; ++k) {
        const Frame& fr = frames[k];
        const int fi = fr.index >= 0 ? fr.index : first_index + k;
        if (fr.rank < 0 || fr.rank >= nprocs) throw Error(1, "frame rank outside the run's rank count");
        if (k > 0 && fr.rank != frames[k - 1].rank) small = false;   // each rank has its own neighbour lists
        if (fr.natoms <= 0) throw Error(2, "frame with no atoms");
        if (fr.natoms > 8191) throw Error(2, "frames above 8191 atoms are not supported on the device");
        RowLayout rl = frame_rows(m, fi, fr.natoms);
        fb.natoms.push_back(fr.natoms);
        fb.stress_rows.push_back(rl.stress_rows);
        fb.energy_rows.push_back(rl.energy_rows);
        fb.atom_ofs.push_back(fb.atom_ofs.back() + fr.natoms);
        fb.ghost_ofs.push_back(fb.ghost_ofs.back() + (int64_t)nimg * fr.natoms);
        fb.row_ofs.push_back(fb.row_ofs.back() + rl.total());
        small = frame_is_small(m, fr.box, small);
        fb.small_self.push_back(frame_is_small(m, fr.box, false) ? 1 : 0);
        fb.file.push_back(fr.file);
        fb.rank.push_back(fr.rank);
        cgd::BoxDev bd;
        std::memset(&bd, 0, sizeof(bd));
        for (int q = 0; q < 9; ++q) { bd.h[q] = fr.box.hmat[q]; bd.inv[q] = fr.box.invr[q]; }
        bd.lx = fr.box.lx; bd.ly = fr.box.ly; bd.lz = fr.box.lz; bd.vol = fr.box.vol;
        bd.is_ortho = fr.box.is_ortho ? 1 : 0;
        bd.small = small ? 1 : 0;
        set_small(bd, small);
        if (m.ncoul > 0 || m.ctl.use_partial_charges) {   // optimal_ewald_params (orthorhombic cells only)
            if (!fr.box.is_ortho) throw Error(2, "the Ewald charge columns need an orthorhombic cell");
            const EwaldParams ep = ewald_params(fr.natoms, fr.box);
            bd.ew_alpha = ep.alpha; bd.ew_rc = ep.rc; bd.ew_kmax = ep.kmax;
        }
        fb.box.push_back(bd);
        fb.type.insert(fb.type.end(), fr.type.begin(), fr.type.end());
        fb.xyz.insert(fb.xyz.end(), fr.xyz.begin(), fr.xyz.end());
        for (int a = 0; a < fr.natoms; ++a)
            for (int q = 0; q < 3; ++q) fb.b.push_back(fr.force[3 * a + q]);
        if (rl.stress_rows == 3) {
            for (int q = 0; q < 3; ++q) fb.b.push_back(fr.stress_diag[q] / GPA);
        } else if (rl.stress_rows == 9) {
            const double xx = fr.stress_diag[0], yy = fr.stress_diag[1], zz = fr.stress_diag[2];
            const double xy = fr.stress_off[0], xz = fr.stress_off[1], yz = fr.stress_off[2];
            const double v[9] = {xx, xy, xz, xy, yy, yz, xz, yz, zz};
            for (double x : v) fb.b.push_back(x / GPA);
        }
        for (int q = 0; q < rl.energy_rows; ++q) fb.b.push_back(fr.energy);
    }
    fb.nrows = fb.row_ofs.back();
    fb.natoms_total = fb.atom_ofs.back();
    fb.nghosts = fb.ghost_ofs.back();
    return fb;
}

DeviceFrames::~DeviceFrames() {
    for (void* p : allocs) cudaFree(p);
}

}  // namespace cg

namespace cgd {
// ------------------------------------------------------------------ device helpers
__global__ void k_scan_counts(const int* cnt, int n, int64_t* ofs) {
    __shared__ int64_t part[1024];
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(n, b + per);
    int64_t s = 0;
    for (int i = b; i < e; ++i) s += cnt[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        int64_t v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int64_t run = part[threadIdx.x] - s;
    for (int i = b; i < e; ++i) { ofs[i] = run; run += cnt[i]; }
    if (threadIdx.x == blockDim.x - 1) ofs[n] = part[threadIdx.x];
}

__global__ void k_gather_frame_ofs(const int64_t* ofs, const int64_t* atom_ofs, int nframes, int64_t* out) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f <= nframes) out[f] = ofs[atom_ofs[f]];
}

__global__ void k_key_frame_ofs(const int64_t* atom_ofs, int nframes, int per_type, int64_t* out) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f > nframes) return;
    out[f] = per_type > 0 ? (int64_t)f * (per_type + 1) : atom_ofs[f] + f;
}

void launch_scan_counts(const int* cnt, int n, int64_t* ofs, cudaStream_t st) {
    k_scan_counts<<<1, 1024, 0, st>>>(cnt, n, ofs);
}
void launch_gather_frame_ofs(const int64_t* ofs, const int64_t* atom_ofs, int nframes, int64_t* out, cudaStream_t st) {
    k_gather_frame_ofs<<<(nframes + 128) / 128, 128, 0, st>>>(ofs, atom_ofs, nframes, out);
}
void launch_key_frame_ofs(const int64_t* atom_ofs, int nframes, int per_type, int64_t* out, cudaStream_t st) {
    k_key_frame_ofs<<<(nframes + 128) / 128, 128, 0, st>>>(atom_ofs, nframes, per_type, out);
}
}  // namespace cgd

namespace cg {

// ------------------------------------------------------------------ stage timing
static_assert(ST_GRAM_ATB == 11 && ST_GRAM_SPLIT == 12 && ST_GRAM_TC == 13 && ST_GRAM_SYRK == 14,
              "gram.cu brackets its launches with these stage ids");

const char* stage_name(int s) {
    static const char* names[ST_COUNT] = {"frame_setup", "neighbour_lists", "clusters", "buckets", "force_2b",
                                          "virial_2b", "force_3b", "virial_3b", "force_4b", "virial_4b", "other", "gram_atb", "gram_split", "gram_tensor", "gram_fp64_syrk",
                                          "refine_products", "refine_preconditioner", "host_copies"};
    return s >= 0 && s < ST_COUNT ? names[s] : "?";
}

void Session::mark(int stage, bool begin) {
    if (!profiling_) return;
    auto get_event = [&]() {
        cudaEvent_t e;
        if (!event_pool_.empty()) { e = event_pool_.back(); event_pool_.pop_back(); }
        else CK(cudaEventCreate(&e));
        return e;
    };
    if (begin) {
        open_event_ = get_event();
        open_stage_ = stage;
        CK(cudaEventRecord(open_event_, stream_));
    } else if (open_stage_ == stage) {
        cudaEvent_t e = get_event();
        CK(cudaEventRecord(e, stream_));
        pending_.push_back({stage, open_event_, e});
        open_stage_ = -1;
    }
}

void Session::stage_totals(double* ms, int64_t* calls) {
    for (auto& p : pending_) {
        CK(cudaEventSynchronize(p.b));
        float t = 0.f;
        CK(cudaEventElapsedTime(&t, p.a, p.b));
        stage_ms_[p.stage] += t;
        stage_calls_[p.stage] += 1;
        event_pool_.push_back(p.a);
        event_pool_.push_back(p.b);
    }
    pending_.clear();
    for (int k = 0; k < ST_COUNT; ++k) { if (ms) ms[k] = stage_ms_[k]; if (calls) calls[k] = stage_calls_[k]; }
}

void Session::reset_stage_totals() {
    stage_totals(nullptr, nullptr);
    for (int k = 0; k < ST_COUNT; ++k) { stage_ms_[k] = 0; stage_calls_[k] = 0; }
}

// ------------------------------------------------------------------ session
cudaMemPool_t scratch_pool(int device) {
    static std::mutex mu;
    static std::vector<cudaMemPool_t> pools;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)pools.size() <= device) pools.resize(device + 1, nullptr);
    if (!pools[device]) {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = device;
        cudaMemPool_t pool = nullptr;
        CK(cudaMemPoolCreate(&pool, &props));
        uint64_t keep = uint64_t(32) << 30;
        CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        pools[device] = pool;
    }
    return pools[device];
}

void scratch_pool_trim(int device) { CK(cudaMemPoolTrimTo(scratch_pool(device), 0)); }

Session::Session(const Model& m, int device) : model_(m), device_(device) {
    CK(cudaSetDevice(device));
    // A blocking stream: work the caller queued on the legacy default stream (for
    // example the zeroing of G by a framework) completes before the session's next
    // launch, and the other way round.
    CK(cudaStreamCreateWithFlags(&stream_, cudaStreamDefault));
    CK(cudaDeviceGetAttribute(&sms_, cudaDevAttrMultiProcessorCount, device));
    dm_.reset(new DeviceModel(model_, cgd::VIR_PPT * cgd::MB_THREADS));
}

namespace {
// Host staging for device-to-host row blocks: cudaMallocHost (registered = false), or,
// with huge_pages, memory aligned to 512 MiB, advised for transparent huge pages and
// faulted in before it is registered with CUDA (falling back to cudaMallocHost when
// registration fails).  Measured in a process that had run device-resident assemblies
// first: 8 GB blocks copied into cudaMallocHost memory at 168-186 GB/s from the first
// call on, into the registered memory at 39-40 GB/s in the call that allocated it and
// 159-175 GB/s after (the kernel granted huge pages for only 20-53% of one buffer).
void* staging_alloc(size_t bytes, bool& registered, bool huge_pages) {
    constexpr size_t kAlign = size_t(512) << 20;
    const size_t sz = (bytes + kAlign - 1) / kAlign * kAlign;
    registered = false;
    void* p = huge_pages ? std::aligned_alloc(kAlign, sz) : nullptr;
    if (p) {
        madvise(p, sz, MADV_HUGEPAGE);
        for (size_t o = 0; o < sz; o += 4096) static_cast<volatile char*>(p)[o] = 0;
        if (cudaHostRegister(p, sz, cudaHostRegisterDefault) == cudaSuccess) {
            registered = true;
            return p;
        }
        cudaGetLastError();   // clear the failed registration
        std::free(p);
    }
    void* q = nullptr;
    CK(cudaMallocHost(&q, bytes));
    return q;
}
void staging_free(void* p, bool registered) {
    if (!p) return;
    if (registered) {
        cudaHostUnregister(p);
        std::free(p);
    } else {
        cudaFreeHost(p);
    }
}
}  // namespace

Session::~Session() {
    for (auto& p : pending_) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : event_pool_) cudaEventDestroy(e);
    md_.reset();
    dm_.reset();
    if (side_event_) cudaEventDestroy(side_event_);
    for (int k = 0; k < 2; ++k) {
        if (md_side_[k]) cudaStreamDestroy(md_side_[k]);
        if (md_join_[k]) cudaEventDestroy(md_join_[k]);
    }
    if (md_fork_) cudaEventDestroy(md_fork_);
    if (side_stream_) cudaStreamDestroy(side_stream_);
    if (copy_stream_) cudaStreamDestroy(copy_stream_);
    for (int i = 0; i < 2; ++i) staging_free(pinned_[i], pinned_reg_[i]);
    if (mailbox_host_) cudaFreeHost(mailbox_host_);
    if (stream_) cudaStreamDestroy(stream_);
}

std::unique_ptr<DeviceFrames> Session::upload(const FrameBatch& fb) {
    CK(cudaSetDevice(device_));
    std::unique_ptr<DeviceFrames> df(new DeviceFrames());
    df->nframes = fb.nframes;
    df->nrows = fb.nrows;
    df->natoms_total = fb.natoms_total;
    df->nghosts = fb.nghosts;
    df->atom_ofs_host = fb.atom_ofs;
    df->row_ofs_host = fb.row_ofs;
    df->box_host = fb.box;
    df->natoms_host = fb.natoms;
    cgd::FramesDev& d = df->dev;
    const int L = model_.ctl.nlayers;
    d.nframes = fb.nframes;
    d.nlayers = L;
    d.nimg = (2 * L + 1) * (2 * L + 1) * (2 * L + 1);
    d.natoms = dev_upload(df->allocs, fb.natoms.data(), fb.natoms.size());
    d.atom_ofs = dev_upload(df->allocs, fb.atom_ofs.data(), fb.atom_ofs.size());
    d.ghost_ofs = dev_upload(df->allocs, fb.ghost_ofs.data(), fb.ghost_ofs.size());
    d.row_ofs = dev_upload(df->allocs, fb.row_ofs.data(), fb.row_ofs.size());
    d.stress_rows = dev_upload(df->allocs, fb.stress_rows.data(), fb.stress_rows.size());
    d.energy_rows = dev_upload(df->allocs, fb.energy_rows.data(), fb.energy_rows.size());
    d.box = dev_upload(df->allocs, fb.box.data(), fb.box.size());
    d.type = dev_upload(df->allocs, fb.type.data(), fb.type.size());
    df->xyz = dev_upload(df->allocs, fb.xyz.data(), fb.xyz.size());
    d.xyz = df->xyz;
    double* scaled = nullptr;
    float* c32 = nullptr;
    CK(cudaMalloc((void**)&scaled, std::max<int64_t>(1, fb.nghosts) * 3 * sizeof(double)));
    df->allocs.push_back(scaled);
    CK(cudaMalloc((void**)&c32, std::max<int64_t>(1, fb.nghosts) * 4 * sizeof(float)));
    df->allocs.push_back(c32);
    d.scaled = scaled;
    d.cart32 = c32;
    return df;
}

namespace {
// Largest per-cluster basis table (bytes) an assembly call allocates; bigger
// batches evaluate the bases inside the force and stress kernels instead.
constexpr size_t kClusterBasisMax = size_t(16) << 30;

// Scratch of the no-allocation entry point: one fixed array per device that loads
// this library, held until the process exits.  Host code must not use the symbol
// as an address; noalloc_scratch() obtains the device address once per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[CG_NOALLOC_SCRATCH_BYTES];

void* noalloc_scratch(int device) {
    static std::mutex mu;
    static std::vector<void*> ptr;
    std::lock_guard<std::mutex> lock(mu);
    if ((int)ptr.size() <= device) ptr.resize(device + 1, nullptr);
    if (!ptr[device]) {
        // the caller has made `device` current
        void* p = nullptr;
        cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (rc != cudaSuccess || p == nullptr)
            throw Error(3, std::string("cudaGetSymbolAddress(no-allocation scratch): ") + cudaGetErrorString(rc));
        ptr[device] = p;
    }
    return ptr[device];
}

__global__ void k_count_evals(const int* type, int64_t n, const cgd::ClusterTypeDev* types,
                              unsigned long long* out) {
    unsigned long long local = 0;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
        local += (unsigned long long)types[type[q]].n_allowed;
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(out, local);
}
}  // namespace

void Session::assemble(const DeviceFrames& df, int precision, void* A, int64_t lda, AssembleStats* stats) {
    CK(cudaSetDevice(device_));
    Scratch S(stream_);
    run(df, precision, A, lda, stats, S, nullptr, nullptr);
}

namespace {
constexpr int kMailboxBytes = 256;
struct PeekList {
    const void* src[4];
    int bytes[4];
    int n;
};
__global__ void k_peek(PeekList L, unsigned char* dst) {
    int off = 0;
    for (int i = 0; i < L.n; ++i) {
        const unsigned char* s = static_cast<const unsigned char*>(L.src[i]);
        for (int b = 0; b < L.bytes[i]; ++b) dst[off + b] = s[b];
        off += L.bytes[i];
    }
}
}  // namespace

void Session::peek(cudaStream_t st, std::initializer_list<PeekItem> items) {
    if (!mailbox_host_) {
        CK(cudaHostAlloc((void**)&mailbox_host_, kMailboxBytes, cudaHostAllocMapped));
        CK(cudaHostGetDevicePointer((void**)&mailbox_dev_, mailbox_host_, 0));
    }
    PeekList L{};
    int total = 0;
    for (const PeekItem& it : items) {
        if (L.n == 4 || it.bytes < 0 || total + it.bytes > kMailboxBytes) throw Error(1, "peek list too large");
        L.src[L.n] = it.dev;
        L.bytes[L.n++] = it.bytes;
        total += it.bytes;
    }
    k_peek<<<1, 1, 0, st>>>(L, mailbox_dev_);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    int off = 0;
    for (const PeekItem& it : items) {
        std::memcpy(it.host, mailbox_host_ + off, it.bytes);
        off += it.bytes;
    }
}

void Session::set_host_staging(int kind) {
    const bool huge = kind == 0;
    if (huge == staging_huge_) return;
    staging_huge_ = huge;
    for (int i = 0; i < 2; ++i) {   // the next streamed call allocates the new kind
        staging_free(pinned_[i], pinned_reg_[i]);
        pinned_[i] = nullptr;
        pinned_bytes_[i] = 0;
        pinned_reg_[i] = false;
    }
}

void* Session::pinned(int i, size_t bytes) {
    if (i < 0 || i > 1) throw Error(1, "pinned staging index");
    if (pinned_bytes_[i] < bytes) {
        staging_free(pinned_[i], pinned_reg_[i]);
        pinned_[i] = nullptr;
        pinned_bytes_[i] = 0;
        pinned_[i] = staging_alloc(bytes, pinned_reg_[i], staging_huge_);
        pinned_bytes_[i] = bytes;
    }
    return pinned_[i];
}

int64_t Session::assemble_to_host(const FrameBatch& fb, int precision, int block_frames, int64_t ldh,
                                  const std::function<void*(int64_t, int64_t)>& dest,
                                  const std::function<bool(int64_t, int64_t, const void*)>& done,
                                  AssembleStats* stats) {
    CK(cudaSetDevice(device_));
    const int nf = fb.nframes;
    if (nf == 0) return 0;
    const int bf = std::max(1, std::min(block_frames, nf));
    const int nblk = (nf + bf - 1) / bf;
    const size_t rsz = precision == 0 ? sizeof(double) : sizeof(float);
    if (ldh < model_.tot_all) throw Error(1, "host lda smaller than the number of A columns");
    if (!copy_stream_) CK(cudaStreamCreateWithFlags(&copy_stream_, cudaStreamNonBlocking));
    // every block's frames on the device first (positions and boxes are small)
    std::vector<std::unique_ptr<DeviceFrames>> dev(nblk);
    int64_t maxrows = 1;
    for (int k = 0; k < nblk; ++k) {
        dev[k] = upload(slice_batch(fb, k * bf, std::min(bf, nf - k * bf)));
        maxrows = std::max<int64_t>(maxrows, dev[k]->nrows);
    }
    struct Res {
        void* dA[2] = {nullptr, nullptr};
        cudaEvent_t asm_done[2] = {nullptr, nullptr}, copy_done[2] = {nullptr, nullptr};
        cudaEvent_t copy_t0[2] = {nullptr, nullptr}, copy_t1[2] = {nullptr, nullptr};   // profiling only
        ~Res() {
            for (int i = 0; i < 2; ++i) {
                if (dA[i]) cudaFree(dA[i]);
                if (asm_done[i]) cudaEventDestroy(asm_done[i]);
                if (copy_done[i]) cudaEventDestroy(copy_done[i]);
                if (copy_t0[i]) cudaEventDestroy(copy_t0[i]);
                if (copy_t1[i]) cudaEventDestroy(copy_t1[i]);
            }
        }
    } R;
    const int64_t lda = model_.tot_all;
    for (int i = 0; i < 2 && i < nblk; ++i) CK(cudaMalloc(&R.dA[i], (size_t)maxrows * lda * rsz));
    for (int i = 0; i < 2; ++i) {
        CK(cudaEventCreateWithFlags(&R.asm_done[i], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&R.copy_done[i], cudaEventDisableTiming));
        if (profiling_) {   // the device time of each block's copy to the host (stage host_copies)
            CK(cudaEventCreate(&R.copy_t0[i]));
            CK(cudaEventCreate(&R.copy_t1[i]));
        }
    }
    std::vector<int64_t> first(nblk + 1, 0);
    for (int k = 0; k < nblk; ++k) first[k + 1] = first[k] + dev[k]->nrows;
    std::vector<void*> hdst(nblk, nullptr);
    AssembleStats total, one;
    auto finish = [&](int k) {   // block k's copy has been issued: wait for it, hand it over
        CK(cudaEventSynchronize(R.copy_done[k % 2]));
        if (profiling_) {
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, R.copy_t0[k % 2], R.copy_t1[k % 2]));
            stage_ms_[ST_HOST_COPY] += ms;
            ++stage_calls_[ST_HOST_COPY];
        }
        return done(first[k], dev[k]->nrows, hdst[k]);
    };
    bool go = true;
    for (int k = 0; k < nblk && go; ++k) {
        const int b = k % 2;
        if (k >= 2) CK(cudaStreamWaitEvent(stream_, R.copy_done[b], 0));   // buffer b is free again
        assemble(*dev[k], precision, R.dA[b], lda, stats ? &one : nullptr);
        if (stats) {
            total.pairs2 += one.pairs2; total.list3 += one.list3; total.list4 += one.list4;
            total.triplets += one.triplets; total.quads += one.quads;
            total.power_evals3 += one.power_evals3; total.power_evals4 += one.power_evals4;
            total.launches += one.launches;
        }
        CK(cudaEventRecord(R.asm_done[b], stream_));
        CK(cudaStreamWaitEvent(copy_stream_, R.asm_done[b], 0));
        hdst[k] = dest(first[k], dev[k]->nrows);
        if (!hdst[k]) throw Error(1, "no host destination for a row block");
        if (profiling_) CK(cudaEventRecord(R.copy_t0[b], copy_stream_));
        if (ldh == lda) {
            CK(cudaMemcpyAsync(hdst[k], R.dA[b], (size_t)dev[k]->nrows * lda * rsz, cudaMemcpyDeviceToHost,
                               copy_stream_));
        } else {
            CK(cudaMemcpy2DAsync(hdst[k], (size_t)ldh * rsz, R.dA[b], (size_t)lda * rsz, (size_t)lda * rsz,
                                 (size_t)dev[k]->nrows, cudaMemcpyDeviceToHost, copy_stream_));
        }
        if (profiling_) CK(cudaEventRecord(R.copy_t1[b], copy_stream_));
        CK(cudaEventRecord(R.copy_done[b], copy_stream_));
        if (k >= 1) go = finish(k - 1);
    }
    if (go) finish(nblk - 1);
    CK(cudaStreamSynchronize(copy_stream_));
    CK(cudaStreamSynchronize(stream_));
    if (stats) *stats = total;
    return first[nblk];
}

void Session::assemble_noalloc(const DeviceFrames& df, int precision, void* A, int64_t lda, AssembleStats* stats) {
    CK(cudaSetDevice(device_));
    if (profiling_) throw Error(1, "stage profiling is not available in the no-allocation call");
    Scratch S(stream_, noalloc_scratch(device_), CG_NOALLOC_SCRATCH_BYTES);
    run(df, precision, A, lda, stats, S, nullptr, nullptr);
}

void Session::run(const DeviceFrames& df, int precision, void* A, int64_t lda, AssembleStats* stats, Scratch& S,
                  const RunPlan* plan_in, RunPlan* plan_out) {
    const cgd::ModelDev& M = dm_->dev;
    const cgd::FramesDev& F = df.dev;
    const Model& model = model_;
    cudaStream_t st = stream_;
    const int nf = df.nframes;
    const int nreal = (int)df.natoms_total;
    const int prec = precision;
    const int rsize = prec == 0 ? 8 : 4;
    int64_t launches = 0;
    if (lda < M.tot_all) throw Error(1, "lda smaller than the number of A columns");
    if (nf == 0) return;
    auto L = [&](int n = 1) { launches += n; };
    // ghosts
    mark(ST_SETUP, true);
    cgd::launch_frame_setup(F, df.nghosts, st); L();
    CK(cudaGetLastError());
    mark(ST_SETUP, false);
    // neighbour lists
    mark(ST_NEIGH, true);
    cgd::NeighDev NB{};
    NB.n_real = nreal;
    NB.cnt2 = S.get<int>(nreal); NB.cnt3 = S.get<int>(nreal); NB.cnt4 = S.get<int>(nreal);
    NB.ofs2 = S.get<int64_t>(nreal + 1); NB.ofs3 = S.get<int64_t>(nreal + 1); NB.ofs4 = S.get<int64_t>(nreal + 1);
    cgd::launch_neigh(M, F, NB, 0, st); L();
    cgd::k_scan_counts<<<1, 1024, 0, st>>>(NB.cnt2, nreal, NB.ofs2); L();
    cgd::k_scan_counts<<<1, 1024, 0, st>>>(NB.cnt3, nreal, NB.ofs3); L();
    cgd::k_scan_counts<<<1, 1024, 0, st>>>(NB.cnt4, nreal, NB.ofs4); L();
    int64_t tot[3] = {0, 0, 0};
    if (plan_in) {   // sizes known from an earlier pass: no host synchronisation (capturable)
        for (int k = 0; k < 3; ++k) tot[k] = plan_in->tot[k];
    } else {
        peek(st, {{&tot[0], NB.ofs2 + nreal, 8}, {&tot[1], NB.ofs3 + nreal, 8}, {&tot[2], NB.ofs4 + nreal, 8}});
    }
    if (plan_out) for (int k = 0; k < 3; ++k) plan_out->tot[k] = tot[k];
    NB.i2 = S.get<int>(tot[0]); NB.g2 = S.get<int>(tot[0]); NB.pt2 = S.get<int>(tot[0]);
    NB.r2 = S.get<double>(tot[0]); NB.rab2 = S.get<double>(3 * tot[0]);
    NB.g3 = S.get<int>(tot[1]); NB.r3 = S.get<double>(tot[1]);
    NB.g4 = S.get<int>(tot[2]); NB.r4 = S.get<double>(tot[2]);
    cgd::launch_neigh(M, F, NB, 1, st); L();
    CK(cudaGetLastError());
    mark(ST_NEIGH, false);
    // clusters
    cgd::ClusterSet CS3{}, CS4{};
    unsigned long long* d_evals = S.get<unsigned long long>(2);
    CK(cudaMemsetAsync(d_evals, 0, 2 * sizeof(unsigned long long), st));
    auto clusters = [&](int nbody, cgd::ClusterSet& CS) -> int64_t {
        CS.cnt = S.get<int>(nreal);
        CS.ofs = S.get<int64_t>(nreal + 1);
        if (cgd::cluster_parts(nreal) > 1) CS.pcnt = S.get<int>((size_t)nreal * cgd::cluster_parts(nreal));
        cgd::launch_clusters(nbody, M, F, NB, CS, 0, st); L();
        cgd::k_scan_counts<<<1, 1024, 0, st>>>(CS.cnt, nreal, CS.ofs); L();
        int64_t n = 0;
        if (plan_in) {
            n = plan_in->ncl[nbody - 3];
        } else {
            peek(st, {{&n, CS.ofs + nreal, 8}});
        }
        if (plan_out) plan_out->ncl[nbody - 3] = n;
        CS.m = S.get<int4>(n);
        CS.type = S.get<int>(n);
        cgd::launch_clusters(nbody, M, F, NB, CS, 1, st); L();
        if (n > 0) {
            k_count_evals<<<(unsigned)std::min<int64_t>(1024, (n + 255) / 256), 256, 0, st>>>(
                CS.type, n, nbody == 3 ? M.types3 : M.types4, d_evals + (nbody - 3)); L();
        }
        CK(cudaGetLastError());
        return n;
    };
    mark(ST_CLUSTERS, true);
    int64_t n3 = M.order3 > 0 ? clusters(3, CS3) : 0;
    int64_t n4 = M.order4 > 0 ? clusters(4, CS4) : 0;
    mark(ST_CLUSTERS, false);
    // zero the batch's rows, then write every non-zero block once
    mark(ST_OTHER, true);
    CK(cudaMemsetAsync(A, 0, (size_t)df.nrows * lda * rsize, st));
    int64_t* kfo_atoms = S.get<int64_t>(nf + 1);
    int64_t* kfo_t3 = S.get<int64_t>(nf + 1);
    int64_t* kfo_t4 = S.get<int64_t>(nf + 1);
    cgd::k_key_frame_ofs<<<(nf + 128) / 128, 128, 0, st>>>(F.atom_ofs, nf, 0, kfo_atoms); L();
    if (M.order3 > 0) { cgd::k_key_frame_ofs<<<(nf + 128) / 128, 128, 0, st>>>(F.atom_ofs, nf, M.ntypes3, kfo_t3); L(); }
    if (M.order4 > 0) { cgd::k_key_frame_ofs<<<(nf + 128) / 128, 128, 0, st>>>(F.atom_ofs, nf, M.ntypes4, kfo_t4); L(); }
    mark(ST_OTHER, false);
    const bool virial = model.ctl.fit_stress || model.ctl.fit_stress_all || model.ctl.fit_ener;
    // ---- 2-body
    if (M.order2 > 0) {
        mark(ST_BUCKET, true);
        int64_t* pfo = S.get<int64_t>(nf + 1);
        cgd::k_gather_frame_ofs<<<(nf + 128) / 128, 128, 0, st>>>(NB.ofs2, F.atom_ofs, nf, pfo); L();
        cgd::Buckets inc2{S.get<int64_t>(nreal + nf), S.get<int>(2 * tot[0])};
        cgd::BucketSpec spec{0, 2, pfo, kfo_atoms, NB.i2, NB.g2, nullptr, nullptr};
        cgd::launch_bucket(nf, F, spec, inc2, st); L();
        mark(ST_BUCKET, false);
        const int ncol = M.npairs * M.order2;
        if (ncol > 8 * cgd::F2_THREADS) throw Error(2, "too many 2-body columns for the device kernel");
        mark(ST_FORCE2, true);
        cgd::launch_force2(prec, nreal, M, F, NB, inc2, kfo_atoms, A, lda, st); L();
        mark(ST_FORCE2, false);
        if (virial) {
            mark(ST_VIRIAL2, true);
            const int nsl = cgd::virial2_slices(nf, tot[0], sms_);
            void* part = S.get<double>((size_t)nf * nsl * 7 * ncol);
            cgd::launch_virial2(prec, nf, nsl, M, F, NB, part, A, lda, st); L(2);
            mark(ST_VIRIAL2, false);
        }
        CK(cudaGetLastError());
    }
    const int ncomp = (model.ctl.fit_stress_all ? 7 : (model.ctl.fit_stress ? 4 : 1));
    auto many_body = [&](int nbody, cgd::ClusterSet& CS, int64_t nq, const int64_t* kfo_types, int ntypes, int ord,
                         int max_allowed) {
        if (nq == 0) return;
        mark(ST_BUCKET, true);
        int64_t* cfo = S.get<int64_t>(nf + 1);
        cgd::k_gather_frame_ofs<<<(nf + 128) / 128, 128, 0, st>>>(CS.ofs, F.atom_ofs, nf, cfo); L();
        cgd::Buckets inc{S.get<int64_t>(nreal + nf), S.get<int>(nbody * nq)};
        cgd::BucketSpec spec{1, nbody, cfo, kfo_atoms, nullptr, nullptr, CS.m, nullptr};
        cgd::launch_bucket(nf, F, spec, inc, st); L();
        cgd::Buckets byt{S.get<int64_t>((int64_t)nf * (ntypes + 1)), S.get<int>(nq)};
        cgd::BucketSpec spec2{2, 1, cfo, kfo_types, nullptr, nullptr, nullptr, CS.type};
        cgd::launch_bucket(nf, F, spec2, byt, st); L();
        mark(ST_BUCKET, false);
        const int ppt = (max_allowed + cgd::MB_THREADS - 1) / cgd::MB_THREADS;
        const int pp = ppt <= 1 ? 1 : (ppt <= 2 ? 2 : 8);
        // range form in FP64, and in FP32 where a type has more powers than the per-power
        // form has threads (with one power per thread that form fits three CTAs per SM)
        const bool range = force_range_ == 2 || (force_range_ == 1 && (prec == 0 || ppt > 1));
        int rg_nt = cgd::rg_max_threads(rsize);
        if (range) {
            std::vector<int> na;
            for (const auto& ct : (nbody == 3 ? model.trips : model.quads).vec) na.push_back(ct.excluded ? 0 : ct.n_allowed);
            rg_nt = cgd::rg_threads(na.data(), (int)na.size(), rsize);
        }
        const size_t force_smem = range ? cgd::mb_range_smem(nbody, ord, ntypes * 4, rg_nt, rsize).total
                                        : cgd::mb_force_smem(nbody, ord, ntypes * 4, max_allowed, rsize).total;
        if (!range && ppt > 8) throw Error(2, "too many allowed powers for the device force kernel");
        if (force_smem > 227 * 1024) throw Error(2, "cluster order too large for the device force kernel");
        mark(nbody == 3 ? ST_FORCE3 : ST_FORCE4, true);
        // slot bases once per cluster (the force kernel meets each cluster once per
        // member, the stress kernel once more); evaluated in place when the fixed
        // no-allocation scratch is in use or the table would pass kClusterBasisMax
        void* pre = nullptr;
        const size_t nbasis = cgd::cluster_basis_count(nbody, ord, nq);
        if (!S.base && nbasis * rsize <= kClusterBasisMax) {
            pre = prec == 0 ? (void*)S.get<double>(nbasis) : (void*)S.get<float>(nbasis);
            cgd::launch_cluster_basis(nbody, prec, nq, M, F, CS, pre, st); L();
        }
        if (range)
            cgd::launch_force_rg(nbody, prec, nreal, rg_nt, force_smem, M, F, CS, inc, kfo_atoms, pre, A, lda, st);
        else
            cgd::launch_force_mb(nbody, prec, pp, nreal, force_smem, M, F, CS, inc, kfo_atoms, pre, A, lda, st,
                                 force4_threads_);
        L();
        mark(nbody == 3 ? ST_FORCE3 : ST_FORCE4, false);
        CK(cudaGetLastError());
        if (virial) {
            cgd::MbVirSmem V = cgd::mb_vir_smem(nbody, ord, cgd::VIR_PPT * cgd::MB_THREADS, rsize);
            if (V.total > 227 * 1024) throw Error(2, "cluster order too large for the device stress/energy kernel");
            const int maxz = (max_allowed + cgd::VIR_PPT * cgd::MB_THREADS - 1) / (cgd::VIR_PPT * cgd::MB_THREADS) + 1;
            int* d_max = S.get<int>(1);
            CK(cudaMemsetAsync(d_max, 0, sizeof(int), st));
            cgd::launch_max_bucket(byt.key_ofs, kfo_types, nf, ntypes, d_max, st); L();
            int hmax = 0;
            if (plan_in) {
                hmax = plan_in->hmax[nbody - 3];
            } else {
                peek(st, {{&hmax, d_max, 4}});
            }
            if (plan_out) plan_out->hmax[nbody - 3] = hmax;
            const int nch = std::max(1, (hmax + cgd::VIR_CLUSTERS - 1) / cgd::VIR_CLUSTERS);
            const auto& cl = nbody == 3 ? model.trips : model.quads;
            int ntrue_max = 1;
            for (const auto& ct : cl.vec) ntrue_max = std::max(ntrue_max, ct.excluded ? 0 : ct.n_true);
            void* part = prec == 0 ? (void*)S.get<double>((size_t)nf * ntypes * nch * 7 * ntrue_max)
                                   : (void*)S.get<float>((size_t)nf * ntypes * nch * 7 * ntrue_max);
            mark(nbody == 3 ? ST_VIRIAL3 : ST_VIRIAL4, true);
            const int vppt = max_allowed <= cgd::MB_THREADS ? 1 : cgd::VIR_PPT;
            cgd::launch_virial_mb(nbody, prec, vppt, nf, ntypes, std::min(maxz, cgd::MAXCHUNK), nch, ntrue_max, V.total, M, F,
                                  CS, byt, kfo_types, ncomp, pre, part, A, lda, st); L(2);
            mark(nbody == 3 ? ST_VIRIAL3 : ST_VIRIAL4, false);
            CK(cudaGetLastError());
        }
    };
    if (M.order3 > 0) many_body(3, CS3, n3, kfo_t3, M.ntypes3, M.order3, dm_->max_allowed3);
    if (M.order4 > 0) many_body(4, CS4, n4, kfo_t4, M.ntypes4, M.order4, dm_->max_allowed4);
    if (M.fit_ener_cols > 0) {
        cgd::launch_energy_cols(prec, nf, M, F, A, lda, st); L();
        CK(cudaGetLastError());
    }
    if (M.ncoul > 0) {   // Ewald charge columns (ZCalc_Ewald_Deriv)
        void* ews = S.get<unsigned char>(cgd::ewald_scratch_bytes(nf, model.ctl.natmtyp));
        mark(ST_OTHER, true);
        cgd::launch_ewald(prec, nf, nreal, M, F, ews, A, lda, st); L(3);
        mark(ST_OTHER, false);
        CK(cudaGetLastError());
    }
    if (stats && !plan_in) {
        unsigned long long ev[2] = {0, 0};
        peek(st, {{ev, d_evals, (int)sizeof(ev)}});
        stats->pairs2 = tot[0]; stats->list3 = tot[1]; stats->list4 = tot[2];
        stats->triplets = n3; stats->quads = n4;
        stats->power_evals3 = (int64_t)ev[0]; stats->power_evals4 = (int64_t)ev[1];
        stats->launches = launches;
    }
}

// ------------------------------------------------------------------ normal equations
namespace {
// Row weights of a weighted fit (chimes_lsq.py --weights, src/chimes_lsq.py:140-149:
// A[i][j] * w[i], b[i] * w[i]): the weighted copy of one row block.
template <typename T>
__global__ void k_weight_rows(const T* A, int64_t lda, int64_t nrows, int ncols, const double* b, const double* w,
                              T* out, double* wb) {
    const int64_t r = blockIdx.x;
    if (r >= nrows) return;
    const double wr = w[r];
    for (int c = threadIdx.x; c < ncols; c += blockDim.x) out[r * lda + c] = T(A[r * lda + c] * wr);
    if (threadIdx.x == 0) wb[r] = b[r] * wr;
}
}  // namespace

int64_t Session::gram_plane_rows(int64_t nrows, int ncols) const {
    const int64_t cpad = (ncols + 127) / 128 * 128;
    const int64_t rows = gram_rows_per_launch_ > 0 ? gram_rows_per_launch_ : (int64_t)(1ull << 30) / (4 * cpad);
    return std::min<int64_t>(nrows, std::max<int64_t>(64, rows));
}

void Session::gram(int prec_in, const void* A, int64_t lda, int64_t nrows, int ncols, const double* b, int mode,
                   double* G, double* h, const double* w) {
    CK(cudaSetDevice(device_));
    Scratch S(stream_);
    if (w && nrows > 0) {   // G += (W A)^T (W A), h += (W A)^T (W b) on a weighted copy of the block
        const size_t esz = prec_in == 0 ? sizeof(double) : sizeof(float);
        void* wa = S.get<unsigned char>((size_t)nrows * lda * esz);
        double* wb = S.get<double>(nrows);
        const unsigned blocks = (unsigned)nrows;
        if (prec_in == 0)
            k_weight_rows<double><<<blocks, 256, 0, stream_>>>((const double*)A, lda, nrows, ncols, b, w, (double*)wa, wb);
        else
            k_weight_rows<float><<<blocks, 256, 0, stream_>>>((const float*)A, lda, nrows, ncols, b, w, (float*)wa, wb);
        CK(cudaGetLastError());
        A = wa;
        b = wb;
    }
    int* d_err = S.get<int>(1);
    CK(cudaMemsetAsync(d_err, 0, sizeof(int), stream_));
    void* planes = nullptr;
    size_t pbytes = 0;
    if (mode == 1) {
        const int64_t rb = gram_plane_rows(nrows, ncols);
        pbytes = gram_plane_bytes(rb, ncols);
        planes = S.get<unsigned char>(pbytes);
    }
    try {
        gram_accumulate(prec_in, A, lda, nrows, ncols, b, mode, G, h, planes, pbytes, d_err, stream_,
                        [this](int stage, bool begin) { mark(stage, begin); }, gram_ctas_per_sm_);
    } catch (const std::runtime_error& e) {
        throw Error(3, e.what());
    }
    int herr = 0;
    peek(stream_, {{&herr, d_err, 4}});
    if (herr) throw Error(3, "tensor-core Gram kernel timed out waiting on its pipeline (code " + std::to_string(herr) + ")");
}

void Session::lars(const double* G, const double* h, int ncols, int64_t nsamples, double alpha, int max_iter,
                   double* x, double* info, int mode, double btb, double max_norm, const char* restart_in,
                   const char* restart_out) {
    CK(cudaSetDevice(device_));
    try {
        lars_lasso(G, h, ncols, nsamples, alpha, max_iter, x, info, stream_, mode, btb, max_norm, restart_in,
                   restart_out);
    } catch (const std::runtime_error& e) {
        throw Error(3, e.what());
    }
}

void Session::dlars_normalized(const double* G, const double* h, const double* colsum, double bsum, int ncols,
                               int64_t nsamples, double btb, double lambda, int lasso, int max_iter, double* x,
                               double* info, double max_norm, const char* restart_in, const char* restart_out) {
    CK(cudaSetDevice(device_));
    try {
        cg::dlars_normalized(G, h, colsum, bsum, ncols, nsamples, btb, lambda, lasso, max_iter, x, info, stream_,
                             max_norm, restart_in, restart_out);
    } catch (const std::runtime_error& e) {
        throw Error(2, e.what());
    }
}

void Session::gram_finish(double* G, int ncols) {
    CK(cudaSetDevice(device_));
    gram_symmetrize(G, ncols, true, stream_);
}

void Session::solve(const double* G, const double* h, int ncols, double ridge, const double* A, int64_t lda,
                    int64_t nrows, const double* b, int iters, double* x, double* info) {
    CK(cudaSetDevice(device_));
    Scratch S(stream_);
    double* L = S.get<double>((size_t)ncols * ncols);
    int* d_info = S.get<int>(1);
    try {
        const double used = factor_ridge(G, ncols, ridge, L, d_info, stream_, chol_tensor_);
        if (used < 0.0) throw Error(2, "the normal-equations matrix is not positive definite even with a ridge");
        cholesky_solve64(L, ncols, h, x, stream_);
        PcgStats ps;
        if (iters > 0 && A && b) {
            // preconditioned CG on the FP64 ridge system with products through the resident A
            double* t = S.get<double>(nrows);
            double* partial = S.get<double>(atb_partial_doubles(nrows, ncols));
            Fp64Operator op;
            op.apply = [&](const double* p, double* q) {
                gemv_rows64(A, lda, nrows, ncols, p, nullptr, nullptr, t, stream_);
                CK(cudaMemsetAsync(q, 0, sizeof(double) * ncols, stream_));
                gemv_cols64(A, lda, nrows, ncols, t, q, partial, stream_);
            };
            op.residual = [&](const double* xv, double* r) {
                gemv_rows64(A, lda, nrows, ncols, xv, b, nullptr, t, stream_);
                CK(cudaMemsetAsync(r, 0, sizeof(double) * ncols, stream_));
                gemv_cols64(A, lda, nrows, ncols, t, r, partial, stream_);
            };
            ps = pcg_ridge(L, ncols, ridge, op, x, iters, 1e-15, stream_);
        }
        CK(cudaStreamSynchronize(stream_));
        if (info) { info[0] = ps.rnorm0; info[1] = ps.rnorm; info[2] = used; }
    } catch (const std::runtime_error& e) {
        if (dynamic_cast<const Error*>(&e)) throw;
        throw Error(3, e.what());
    }
}

double Session::fp64_fma_tflops() {
    CK(cudaSetDevice(device_));
    try {
        return cg::fp64_fma_tflops(stream_);
    } catch (const std::runtime_error& e) {
        throw Error(3, e.what());
    }
}

double Session::factor(const double* G, int ncols, double ridge, double* L) {
    CK(cudaSetDevice(device_));
    Scratch S(stream_);
    int* d_info = S.get<int>(1);
    try {
        const double used = factor_ridge(G, ncols, ridge, L, d_info, stream_, chol_tensor_);
        if (used < 0.0) throw Error(2, "the normal-equations matrix is not positive definite even with a ridge");
        return used;
    } catch (const std::runtime_error& e) {
        if (dynamic_cast<const Error*>(&e)) throw;
        throw Error(3, e.what());
    }
}

void Session::factor_solve(const double* L, int ncols, const double* h, double* x) {
    CK(cudaSetDevice(device_));
    try {
        cholesky_solve64(L, ncols, h, x, stream_);
        CK(cudaStreamSynchronize(stream_));
    } catch (const std::runtime_error& e) {
        if (dynamic_cast<const Error*>(&e)) throw;
        throw Error(3, e.what());
    }
}

namespace {
// One pass over every row block: the block's FP64 rows (assembled again into Ablk,
// or kept from an earlier pass in `kept`), t = (b -) A v (t *= w^2), then
// out += A^T t.  Blocks are kept resident while the cache budget allows, so that
// later passes assemble only the others.
struct StreamRows {
    Session& se;
    int ncols;
    const std::vector<const DeviceFrames*>& blocks;
    const std::vector<const double*>& labels;
    const std::vector<const double*>& weights;
    const double *extra_A, *extra_b, *extra_w;
    int64_t extra_rows;
    double *Ablk, *t, *partial;
    int64_t cache_left = 0;            // bytes still allowed for kept blocks
    std::vector<double*> kept;         // per block: resident FP64 rows, or null
    ~StreamRows() { for (double* p : kept) if (p) cudaFree(p); }
    const double* rows_of(size_t k, cudaStream_t st) {
        const DeviceFrames& d = *blocks[k];
        if (kept.size() < blocks.size()) kept.resize(blocks.size(), nullptr);
        if (kept[k]) return kept[k];
        const int64_t bytes = d.nrows * (int64_t)ncols * (int64_t)sizeof(double);
        if (bytes <= cache_left) {
            double* p = nullptr;
            if (cudaMalloc(&p, (size_t)bytes) == cudaSuccess) {
                se.assemble(d, 0, p, ncols, nullptr);
                kept[k] = p;
                cache_left -= bytes;
                return p;
            }
            cudaGetLastError();   // out of memory: assemble into the block buffer instead
            cache_left = 0;
        }
        se.assemble(d, 0, Ablk, ncols, nullptr);
        return Ablk;
    }
    void pass(const double* v, bool resid, double* out, cudaStream_t st) {
        CK(cudaMemsetAsync(out, 0, sizeof(double) * ncols, st));
        for (size_t k = 0; k < blocks.size(); ++k) {
            const DeviceFrames& d = *blocks[k];
            if (d.nrows == 0) continue;
            const double* Ak = rows_of(k, st);
            se.mark(ST_REFINE_PRODUCTS, true);
            gemv_rows64(Ak, ncols, d.nrows, ncols, v, resid ? labels[k] : nullptr,
                        weights.empty() ? nullptr : weights[k], t, st);
            gemv_cols64(Ak, ncols, d.nrows, ncols, t, out, partial, st);
            se.mark(ST_REFINE_PRODUCTS, false);
        }
        if (extra_rows > 0) {
            gemv_rows64(extra_A, ncols, extra_rows, ncols, v, resid ? extra_b : nullptr, extra_w, t, st);
            gemv_cols64(extra_A, ncols, extra_rows, ncols, t, out, partial, st);
        }
    }
};
}  // namespace

void Session::refine_streamed(const double* L, int ncols, double ridge, const std::vector<const DeviceFrames*>& blocks,
                              const std::vector<const double*>& labels, const std::vector<const double*>& weights,
                              const double* extra_A, int64_t extra_rows, const double* extra_b, const double* extra_w,
                              int max_iters, double tol, double* x, double* info) {
    CK(cudaSetDevice(device_));
    if (blocks.size() != labels.size() || (!weights.empty() && weights.size() != blocks.size()))
        throw Error(1, "blocks, labels and weights differ in number");
    if (ncols != model_.tot_all) throw Error(1, "ncols is not the model's column count");
    Scratch S(stream_);
    int64_t maxrows = std::max<int64_t>(1, extra_rows);
    for (const DeviceFrames* d : blocks) maxrows = std::max<int64_t>(maxrows, d->nrows);
    StreamRows R{*this, ncols, blocks, labels, weights, extra_A, extra_b, extra_w, extra_rows,
                 S.get<double>((size_t)maxrows * ncols), S.get<double>(maxrows),
                 S.get<double>(atb_partial_doubles(maxrows, ncols))};
    if (refine_cache_bytes_ < 0) {   // what is free now, less a margin for the assembly's own work lists
        size_t fr = 0, tot = 0;
        CK(cudaStreamSynchronize(stream_));
        scratch_pool_trim(device_);
        CK(cudaMemGetInfo(&fr, &tot));
        // margin: a sixteenth of the device plus one more row block, far above the
        // work lists of one block's assembly (a few GB for 50 four-body frames)
        const int64_t margin = (int64_t)(tot / 16) + (int64_t)maxrows * ncols * (int64_t)sizeof(double);
        R.cache_left = std::max<int64_t>(0, (int64_t)fr - margin);
    } else {
        R.cache_left = refine_cache_bytes_;
    }
    try {
        Fp64Operator op;
        op.apply = [&](const double* p, double* q) { R.pass(p, false, q, stream_); };
        op.residual = [&](const double* xv, double* r) { R.pass(xv, true, r, stream_); };
        op.mark = [this](bool begin) { mark(ST_REFINE_PRECOND, begin); };
        const PcgStats ps = pcg_ridge(L, ncols, ridge, op, x, max_iters, tol, stream_);
        CK(cudaStreamSynchronize(stream_));
        if (info) { info[0] = ps.iters; info[1] = ps.rel_update; info[2] = ps.rnorm0; info[3] = ps.rnorm; }
    } catch (const std::runtime_error& e) {
        if (dynamic_cast<const Error*>(&e)) throw;
        throw Error(3, e.what());
    }
}

void Session::solve_streamed(const double* G, const double* h, int ncols, double ridge,
                             const std::vector<const DeviceFrames*>& blocks, const std::vector<const double*>& labels,
                             const std::vector<const double*>& weights, const double* extra_A, int64_t extra_rows,
                             const double* extra_b, const double* extra_w, int max_iters, double tol, double* x,
                             double* info) {
    CK(cudaSetDevice(device_));
    Scratch S(stream_);
    double* L = S.get<double>((size_t)ncols * ncols);
    const double used = factor(G, ncols, ridge, L);
    factor_solve(L, ncols, h, x);
    double in[4] = {0, 0, 0, 0};
    refine_streamed(L, ncols, ridge, blocks, labels, weights, extra_A, extra_rows, extra_b, extra_w, max_iters, tol, x,
                    in);
    if (info) { for (int k = 0; k < 4; ++k) info[k] = in[k]; info[4] = used; }
}

void Session::predict_streamed(const std::vector<const DeviceFrames*>& blocks, const double* x, double* y) {
    CK(cudaSetDevice(device_));
    const int ncols = model_.tot_all;
    Scratch S(stream_);
    int64_t maxrows = 1;
    for (const DeviceFrames* d : blocks) maxrows = std::max<int64_t>(maxrows, d->nrows);
    double* Ablk = S.get<double>((size_t)maxrows * ncols);
    try {
        int64_t r0 = 0;
        for (const DeviceFrames* d : blocks) {
            if (d->nrows == 0) continue;
            assemble(*d, 0, Ablk, ncols, nullptr);
            gemv_rows64(Ablk, ncols, d->nrows, ncols, x, nullptr, nullptr, y + r0, stream_);
            r0 += d->nrows;
        }
        CK(cudaStreamSynchronize(stream_));
    } catch (const std::runtime_error& e) {
        if (dynamic_cast<const Error*>(&e)) throw;
        throw Error(3, e.what());
    }
}

// ------------------------------------------------------------------ batched fit as one graph
RunPlan Session::plan(const DeviceFrames& df, int precision, void* A, int64_t lda) {
    CK(cudaSetDevice(device_));
    RunPlan p;
    Scratch S(stream_);
    run(df, precision, A, lda, nullptr, S, nullptr, &p);
    CK(cudaStreamSynchronize(stream_));
    return p;
}

BatchFit::~BatchFit() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (d_err) cudaFree(d_err);
}

std::unique_ptr<BatchFit> Session::batch_fit_graph(const std::vector<const DeviceFrames*>& blocks,
                                                   const std::vector<RunPlan>& plans,
                                                   const std::vector<const double*>& labels, int precision,
                                                   void* Abuf, int64_t lda, double* G, double* h) {
    CK(cudaSetDevice(device_));
    if (blocks.size() != plans.size() || blocks.size() != labels.size()) throw Error(1, "blocks / plans / labels");
    if (profiling_) throw Error(1, "stage profiling is not available while capturing a graph");
    const Model& m = model_;
    std::unique_ptr<BatchFit> bf(new BatchFit());
    CK(cudaMalloc((void**)&bf->d_err, sizeof(int)));
    CK(cudaMemset(bf->d_err, 0, sizeof(int)));
    const int ncols = m.tot_all;
    int64_t maxrows = 1;
    for (const DeviceFrames* d : blocks) maxrows = std::max<int64_t>(maxrows, d->nrows);
    const int64_t rb = gram_plane_rows(maxrows, ncols);
    const size_t pbytes = gram_plane_bytes(rb, ncols);
    CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeRelaxed));
    try {
        for (size_t k = 0; k < blocks.size(); ++k) {
            Scratch S(stream_);
            run(*blocks[k], precision, Abuf, lda, nullptr, S, &plans[k], nullptr);
            void* planes = S.get<unsigned char>(pbytes);
            gram_accumulate(precision, Abuf, lda, blocks[k]->nrows, ncols, labels[k], 1, G, h, planes, pbytes,
                            bf->d_err, stream_, [](int, bool) {}, gram_ctas_per_sm_);
        }
    } catch (...) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream_, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    CK(cudaStreamEndCapture(stream_, &bf->graph));
    CK(cudaGraphInstantiate(&bf->exec, bf->graph, 0));
    size_t nodes = 0;
    CK(cudaGraphGetNodes(bf->graph, nullptr, &nodes));
    bf->nodes = (int64_t)nodes;
    return bf;
}

void Session::batch_fit_launch(BatchFit& bf) {
    CK(cudaSetDevice(device_));
    CK(cudaGraphLaunch(bf.exec, stream_));
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, bf.d_err, sizeof(int), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    if (herr) throw Error(3, "tensor-core Gram kernel timed out waiting on its pipeline (code " + std::to_string(herr) + ")");
}

}  // namespace cg
