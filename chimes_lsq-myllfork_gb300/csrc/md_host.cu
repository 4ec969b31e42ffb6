// Host orchestration of the MD force and the NVE integrator on one GPU.
//
//   ZCalc             src/functions.C:815-891   -> Session::md_force
//   chimes_md MD loop src/chimes_md.C:700-1050  -> Session::md_nve (NVE only)
//
// The per-step launch sequence is the design-matrix path's enumeration (ghosts,
// neighbour lists, clusters, per-(frame, type) buckets) followed by the force
// kernels of md.cu.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "assemble.h"
#include "kernels.h"
#include "md.h"
#include "scratch.h"
#include "session.h"
#include "md_server.h"

namespace cg {

// Largest Ewald k cut-off of a batch's frames (the k-space scratch is sized by it).
static int md_ewald_kmax(const DeviceFrames& df) {
    int km = 1;
    for (const auto& b : df.box_host) km = std::max(km, b.ew_kmax);
    return km;
}

void Session::md_setup(const double* x, int nx, int precision, bool offsets, double pen_dist, double pen_scale) {
    CK(cudaSetDevice(device_));
    const Model& m = model_;
    if (nx != m.tot_all) throw Error(1, "coefficient count does not match the model's columns");
    if (precision != 0 && precision != 1) throw Error(1, "MD precision must be 0 (FP64) or 1 (FP32 contraction)");
    const int o2 = m.ctl.cheby_order, o3 = m.ctl.use3 ? m.ctl.cheby3 : 0, o4 = m.ctl.use4 ? m.ctl.cheby4 : 0;
    if (o3 > 16) throw Error(2, "3-body order above 16 is not supported by the MD force");
    if (o4 > 6) throw Error(2, "4-body order above 6 is not supported by the MD force");
    if (precision == 1 && ((o3 > 0 && !cgd::md_fast_order(3, o3)) || (o4 > 0 && !cgd::md_fast_order(4, o4))))
        throw Error(2, "the FP32 MD contraction supports 3-body orders 2-8 and 4-body orders 2-4");
    std::unique_ptr<MdTables> t(new MdTables());
    t->precision = precision;
    auto up = [&](const void* src, size_t bytes) {
        void* p = nullptr;
        CK(cudaMalloc(&p, std::max<size_t>(bytes, 8)));
        t->allocs.push_back(p);
        if (bytes) CK(cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice));
        return p;
    };
    // 2-body: x[col_pt + n] multiplies T_{n+1} (src/chimes_lsq.py:462-477 layout);
    // pair types a HIERARC fit excluded keep zero coefficients, as its params.txt prints
    std::vector<double> c2((size_t)m.pairs.size() * o2, 0.0);
    for (size_t pt = 0; pt < m.pairs.size(); ++pt)
        if (m.pairs[pt].col >= 0)
            for (int n = 0; n < o2; ++n) c2[pt * o2 + n] = x[m.pairs[pt].col + n];
    t->dev.c2 = (const double*)up(c2.data(), c2.size() * sizeof(double));
    // dense cluster tensors: C[type][p_0..p_{n-1}] = x[col_type + PARAM_INDICES[q]]
    auto dense = [&](const ClusterList& cl, int np, int ord, int col0, std::vector<double>& out) {
        size_t sz = 1;
        for (int k = 0; k < np; ++k) sz *= (size_t)ord;
        out.assign(cl.vec.size() * sz, 0.0);
        int col = col0;
        for (size_t T = 0; T < cl.vec.size(); ++T) {
            const ClusterType& ct = cl.vec[T];
            if (!ct.excluded) {
                for (int q = 0; q < ct.n_allowed; ++q) {
                    size_t idx = 0;
                    for (int s = 0; s < np; ++s) idx = idx * ord + ct.allowed_powers[q][s];
                    out[T * sz + idx] = x[col + ct.param_indices[q]];
                }
            }
            col += ct.n_true;
        }
    };
    std::vector<double> C3, C4;
    if (o3 > 0) dense(m.trips, 3, o3, m.tot_snum, C3);
    if (o4 > 0) dense(m.quads, 6, o4, m.tot_snum + m.num3, C4);
    t->dev.C3 = (const double*)up(C3.data(), C3.size() * sizeof(double));
    t->dev.C4 = (const double*)up(C4.data(), C4.size() * sizeof(double));
    std::vector<float> C3f(C3.begin(), C3.end()), C4f(C4.begin(), C4.end());
    t->dev.C3f = (const float*)up(C3f.data(), C3f.size() * sizeof(float));
    t->dev.C4f = (const float*)up(C4f.data(), C4f.size() * sizeof(float));
    t->dev.eoff = nullptr;
    if (offsets) {   // HIERARC-excluded types have offset 0
        if (!m.ctl.fit_ener) throw Error(2, "the model has no energy-offset columns");
        std::vector<double> eo(m.ctl.natmtyp, 0.0);
        for (int ty = 0; ty < m.ctl.natmtyp; ++ty)
            if (m.ener_col[ty] >= 0) eo[ty] = x[m.tot_short + m.ncoul + m.ener_col[ty]];
        t->dev.eoff = (const double*)up(eo.data(), eo.size() * sizeof(double));
    }
    // FITCOUL: charges from the fitted products (chimes_md read_ff_params,
    // src/chimes_md.C:2000-2080): q products in Stillinger units over ke, q_t =
    // sign_t sqrt(|q_t q_t|), every pair's product within 1e-4 of q_i q_j
    t->dev.coulomb = 0;
    if (m.ncoul > 0) {
        const double ke = 332.0637157615209;   // src/functions.h:40
        const int nt = m.ctl.natmtyp;
        if (nt > 10) throw Error(2, "Ewald MD supports up to 10 atom types");
        for (int i = 0; i < nt; ++i) {
            const double qq = x[m.tot_short + m.int_pair_map[i * nt + i]] / ke;
            const std::string& sg = m.pairs[i].chrgsgn;
            const double sign = sg.find('-') != std::string::npos ? -1.0 : 1.0;
            t->dev.qtype[i] = std::sqrt(std::fabs(qq)) * sign;
        }
        for (int i = 0; i < nt; ++i)
            for (int j = 0; j < nt; ++j) {
                const double qq = x[m.tot_short + m.int_pair_map[i * nt + j]] / ke;
                if (std::fabs(t->dev.qtype[i] * t->dev.qtype[j] - qq) > 1.0e-4)
                    throw Error(2, "Inconsistent pair charges for pair: " + m.atom_types[i] + m.atom_types[j]);
            }
        t->dev.coulomb = 1;
    } else if (m.ctl.use_partial_charges) {   // fixed charges (ATMCHRG), chimes_md.C:2024-2036
        if (m.ctl.natmtyp > 10) throw Error(2, "Ewald MD supports up to 10 atom types");
        for (int i = 0; i < m.ctl.natmtyp; ++i) t->dev.qtype[i] = m.pairs[i].chg1;
        t->dev.coulomb = 1;
    }
    t->dev.pen_dist = pen_dist;
    t->dev.pen_scale = pen_scale;
    md_ = std::move(t);
}

void Session::md_force(const DeviceFrames& df, double* Fo, double* So, MdCounts* counts) {
    CK(cudaSetDevice(device_));
    if (!md_) throw Error(1, "MD coefficients are not set (cg_md_setup)");
    const cgd::ModelDev& M = dm_->dev;
    const cgd::MdDev& D = md_->dev;
    const cgd::FramesDev& F = df.dev;
    cudaStream_t st = stream_;
    const int nf = df.nframes;
    const int nreal = (int)df.natoms_total;
    MdCounts c;
    auto L = [&](int n = 1) { c.launches += n; };
    CK(cudaMemsetAsync(Fo, 0, std::max<size_t>(1, (size_t)nreal * 3) * sizeof(double), st));
    CK(cudaMemsetAsync(So, 0, std::max<size_t>(1, (size_t)nf * cgd::MD_NSCALAR) * sizeof(double), st));
    if (nf == 0) { if (counts) *counts = c; return; }
    Scratch S(st);
    cgd::launch_frame_setup(F, df.nghosts, st); L();
    cgd::NeighDev NB{};
    NB.n_real = nreal;
    NB.md = 1;
    NB.cnt2 = S.get<int>(nreal); NB.cnt3 = S.get<int>(nreal); NB.cnt4 = S.get<int>(nreal);
    NB.ofs2 = S.get<int64_t>(nreal + 1); NB.ofs3 = S.get<int64_t>(nreal + 1); NB.ofs4 = S.get<int64_t>(nreal + 1);
    cgd::launch_neigh(M, F, NB, 0, st); L();
    cgd::launch_scan_counts(NB.cnt2, nreal, NB.ofs2, st); L();
    cgd::launch_scan_counts(NB.cnt3, nreal, NB.ofs3, st); L();
    cgd::launch_scan_counts(NB.cnt4, nreal, NB.ofs4, st); L();
    int64_t tot[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(&tot[0], NB.ofs2 + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&tot[1], NB.ofs3 + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&tot[2], NB.ofs4 + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    mark(ST_NEIGH, false);
    CK(cudaStreamSynchronize(st));
    mark(ST_NEIGH, true);
    NB.i2 = S.get<int>(tot[0]); NB.g2 = S.get<int>(tot[0]); NB.pt2 = S.get<int>(tot[0]);
    NB.r2 = S.get<double>(tot[0]); NB.rab2 = S.get<double>(3 * tot[0]);
    NB.g3 = S.get<int>(tot[1]); NB.r3 = S.get<double>(tot[1]);
    NB.g4 = S.get<int>(tot[2]); NB.r4 = S.get<double>(tot[2]);
    cgd::launch_neigh(M, F, NB, 1, st); L();
    c.pairs2 = tot[0];
    cgd::launch_md2(M, D, F, NB, Fo, So, st, md_->precision); L();
    CK(cudaGetLastError());
    // clusters: count both body counts, then one host read of the totals
    cgd::ClusterSet CS3{}, CS4{};
    int64_t ncl[2] = {0, 0};
    const bool use[2] = {M.order3 > 0, M.order4 > 0};
    cgd::ClusterSet* css[2] = {&CS3, &CS4};
    for (int k = 0; k < 2; ++k) {
        if (!use[k]) continue;
        css[k]->cnt = S.get<int>(nreal);
        css[k]->ofs = S.get<int64_t>(nreal + 1);
        if (cgd::cluster_parts(nreal) > 1) css[k]->pcnt = S.get<int>((size_t)nreal * cgd::cluster_parts(nreal));
        cgd::launch_clusters(3 + k, M, F, NB, *css[k], 0, st); L();
        cgd::launch_scan_counts(css[k]->cnt, nreal, css[k]->ofs, st); L();
        CK(cudaMemcpyAsync(&ncl[k], css[k]->ofs + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    }
    if (use[0] || use[1]) CK(cudaStreamSynchronize(st));
    c.triplets = ncl[0];
    c.quads = ncl[1];
    for (int k = 0; k < 2; ++k) {
        const int64_t n = ncl[k];
        if (!use[k] || n == 0) continue;
        const int nbody = 3 + k;
        const int ntypes = k == 0 ? M.ntypes3 : M.ntypes4;
        cgd::ClusterSet& CS = *css[k];
        CS.m = S.get<int4>(n);
        CS.type = S.get<int>(n);
        cgd::launch_clusters(nbody, M, F, NB, CS, 1, st); L();
        int64_t* cfo = S.get<int64_t>(nf + 1);
        cgd::launch_gather_frame_ofs(CS.ofs, F.atom_ofs, nf, cfo, st); L();
        cgd::MdBuckets B{};
        B.ntypes = ntypes;
        B.nkeys = nf * ntypes;
        B.start = S.get<int64_t>(B.nkeys + 1);
        B.tile_ofs = S.get<int>(B.nkeys + 1);
        B.cursor = S.get<int>(B.nkeys);
        B.val = S.get<int>(n);
        cgd::launch_md_bucket(n, nf, cfo, CS.type, B, st); L(3);
        const int64_t max_tiles = (n + cgd::MDC_TILE - 1) / cgd::MDC_TILE + B.nkeys;
        cgd::launch_mdc(nbody, md_->precision, k == 0 ? M.order3 : M.order4, max_tiles, M, D, F, CS, B, Fo, So, st);
        L();
        CK(cudaGetLastError());
    }
    if (D.coulomb) {   // ZCalc_Ewald
        const int km = md_ewald_kmax(df);
        void* ews = S.get<unsigned char>(cgd::md_ewald_scratch_bytes(nf, km));
        cgd::launch_md_ewald(nf, nreal, km, M, D, F, ews, Fo, So, st); L(3);
    }
    cgd::launch_md_finalize(nf, M, D, F, So, st); L();
    CK(cudaGetLastError());
    if (counts) *counts = c;
}

void* MdLists::buffer(int slot, size_t bytes) {
    bytes = std::max<size_t>(bytes, 8);
    if ((int)allocs.size() <= slot) { allocs.resize(slot + 1, nullptr); caps.resize(slot + 1, 0); }
    if (caps[slot] < bytes) {
        if (allocs[slot]) CK(cudaFree(allocs[slot]));
        allocs[slot] = nullptr;
        const size_t grown = bytes + bytes / 4;   // room for the next build
        CK(cudaMalloc(&allocs[slot], grown));
        caps[slot] = grown;
    }
    return allocs[slot];
}

MdLists::~MdLists() {
    for (void* p : allocs) if (p) cudaFree(p);
}

void Session::md_lists_build(DeviceFrames& df, double skin, MdLists& L, cudaStream_t st) {
    CK(cudaSetDevice(device_));
    const cgd::ModelDev& M = dm_->dev;
    const bool timed = st == stream_;   // stage marks time the main stream only
    auto mark = [&](int stage, bool begin) { if (timed) this->mark(stage, begin); };
    const int nf = df.nframes;
    const int nreal = (int)df.natoms_total;
    L.release();
    L.skin = skin;
    L.natoms = nreal;
    int slot = 0;
    auto get = [&](size_t bytes) { return L.buffer(slot++, bytes); };
    L.shift = (int*)get(sizeof(int) * 3 * std::max(nreal, 1));
    L.xref = (double*)get(sizeof(double) * 3 * std::max(nreal, 1));
    L.dmax = (unsigned long long*)get(sizeof(unsigned long long));
    L.scaled = (double*)get(sizeof(double) * 3 * std::max<int64_t>(df.nghosts, 1));
    L.cart32 = (float*)get(sizeof(float) * 4 * std::max<int64_t>(df.nghosts, 1));
    CK(cudaMemcpyAsync(L.xref, df.xyz, sizeof(double) * 3 * nreal, cudaMemcpyDeviceToDevice, st));
    cgd::FramesDev F = df.dev;
    F.shift = L.shift;
    F.shift_mode = 1;   // wrap now and remember the shifts
    F.scaled = L.scaled;
    F.cart32 = L.cart32;
    mark(ST_NEIGH, true);
    cgd::launch_frame_setup(F, df.nghosts, st);
    cgd::NeighDev& NB = L.NB;
    NB = cgd::NeighDev{};
    NB.n_real = nreal;
    NB.md = 2;
    NB.skin = skin;
    NB.cnt2 = (int*)get(sizeof(int) * nreal); NB.cnt3 = (int*)get(sizeof(int) * nreal);
    NB.cnt4 = (int*)get(sizeof(int) * nreal);
    NB.ofs2 = (int64_t*)get(sizeof(int64_t) * (nreal + 1)); NB.ofs3 = (int64_t*)get(sizeof(int64_t) * (nreal + 1));
    NB.ofs4 = (int64_t*)get(sizeof(int64_t) * (nreal + 1));
    // binned search: fractional bins at least the search radius wide along each
    // reciprocal direction (width_d = 1 / |row d of H^-1|)
    const Model& mod = model_;
    double rc = mod.max_cutoff_2b;
    if (M.order3 > 0) rc = std::max(rc, mod.max_cutoff_3b);
    if (M.order4 > 0) rc = std::max(rc, mod.max_cutoff_4b);
    rc += skin + 0.02;
    const int Lr = df.dev.nlayers;
    std::vector<cgd::BinGrid> grid(nf);
    int64_t nbins = 0;
    for (int f = 0; f < nf; ++f) {
        const cgd::BoxDev& bx = df.box_host.at(f);
        for (int d = 0; d < 3; ++d) {
            const double* row = bx.inv + 3 * d;
            const double width = 1.0 / std::sqrt(row[0] * row[0] + row[1] * row[1] + row[2] * row[2]);
            grid[f].nb[d] = std::max(1, std::min(256, (int)std::floor((2 * Lr + 1) * width / rc)));
        }
        grid[f].ofs = nbins;
        nbins += (int64_t)grid[f].nb[0] * grid[f].nb[1] * grid[f].nb[2];
    }
    cgd::Bins BN{};
    BN.nbins = nbins;
    cgd::BinGrid* dgrid = (cgd::BinGrid*)get(sizeof(cgd::BinGrid) * nf);
    CK(cudaMemcpyAsync(dgrid, grid.data(), sizeof(cgd::BinGrid) * nf, cudaMemcpyHostToDevice, st));
    BN.grid = dgrid;
    BN.count = (int*)get(sizeof(int) * nbins);
    BN.start = (int64_t*)get(sizeof(int64_t) * (nbins + 1));
    BN.atoms = (int*)get(sizeof(int) * df.nghosts);
    cgd::launch_bins(F, df.nghosts, BN, st);
    cgd::launch_neigh_binned(M, F, NB, BN, 0, st);
    cgd::launch_scan_counts(NB.cnt2, nreal, NB.ofs2, st);
    cgd::launch_scan_counts(NB.cnt3, nreal, NB.ofs3, st);
    cgd::launch_scan_counts(NB.cnt4, nreal, NB.ofs4, st);
    int64_t tot[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(&tot[0], NB.ofs2 + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&tot[1], NB.ofs3 + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&tot[2], NB.ofs4 + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    mark(ST_NEIGH, false);
    CK(cudaStreamSynchronize(st));
    mark(ST_NEIGH, true);
    NB.i2 = (int*)get(sizeof(int) * tot[0]); NB.g2 = (int*)get(sizeof(int) * tot[0]);
    NB.pt2 = (int*)get(sizeof(int) * tot[0]); NB.r2 = (double*)get(sizeof(double) * tot[0]);
    NB.rab2 = (double*)get(sizeof(double) * 3 * tot[0]);
    NB.g3 = (int*)get(sizeof(int) * tot[1]); NB.r3 = (double*)get(sizeof(double) * tot[1]);
    NB.g4 = (int*)get(sizeof(int) * tot[2]); NB.r4 = (double*)get(sizeof(double) * tot[2]);
    cgd::launch_neigh_binned(M, F, NB, BN, 1, st);
    mark(ST_NEIGH, false);
    mark(ST_CLUSTERS, true);
    const bool use[2] = {M.order3 > 0, M.order4 > 0};
    for (int k = 0; k < 2; ++k) {
        if (!use[k]) continue;
        L.CS[k].cnt = (int*)get(sizeof(int) * nreal);
        L.CS[k].ofs = (int64_t*)get(sizeof(int64_t) * (nreal + 1));
        L.CS[k].pcnt = (int*)get(sizeof(int) * (size_t)nreal * cgd::cluster_parts(nreal));
        cgd::launch_clusters(3 + k, M, F, NB, L.CS[k], 0, st);
        cgd::launch_scan_counts(L.CS[k].cnt, nreal, L.CS[k].ofs, st);
        CK(cudaMemcpyAsync(&L.ncl[k], L.CS[k].ofs + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    }
    mark(ST_CLUSTERS, false);
    CK(cudaStreamSynchronize(st));
    mark(ST_CLUSTERS, true);
    for (int k = 0; k < 2; ++k) {
        if (!use[k] || L.ncl[k] == 0) continue;
        const int64_t n = L.ncl[k];
        const int ntypes = k == 0 ? M.ntypes3 : M.ntypes4;
        L.CS[k].m = (int4*)get(sizeof(int4) * n);
        L.CS[k].type = (int*)get(sizeof(int) * n);
        cgd::launch_clusters(3 + k, M, F, NB, L.CS[k], 1, st);
        L.cfo[k] = (int64_t*)get(sizeof(int64_t) * (nf + 1));
        cgd::launch_gather_frame_ofs(L.CS[k].ofs, F.atom_ofs, nf, L.cfo[k], st);
        L.tstep[k] = (int*)get(sizeof(int) * n);
        cgd::MdBuckets& B = L.B[k];
        B.ntypes = ntypes;
        B.nkeys = nf * ntypes;
        B.start = (int64_t*)get(sizeof(int64_t) * (B.nkeys + 1));
        B.tile_ofs = (int*)get(sizeof(int) * (B.nkeys + 1));
        B.cursor = (int*)get(sizeof(int) * B.nkeys);
        B.val = (int*)get(sizeof(int) * n);
    }
    mark(ST_CLUSTERS, false);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    L.valid = true;
    ++L.builds;
}

void Session::md_force_lists(DeviceFrames& df, MdLists& L, double* Fo, double* So) {
    CK(cudaSetDevice(device_));
    if (!md_) throw Error(1, "MD coefficients are not set (cg_md_setup)");
    if (!L.valid) throw Error(1, "MD lists are not built");
    const cgd::ModelDev& M = dm_->dev;
    const cgd::MdDev& D = md_->dev;
    cudaStream_t st = stream_;
    const int nf = df.nframes;
    const int nreal = (int)df.natoms_total;
    CK(cudaMemsetAsync(Fo, 0, std::max<size_t>(1, (size_t)nreal * 3) * sizeof(double), st));
    CK(cudaMemsetAsync(So, 0, std::max<size_t>(1, (size_t)nf * cgd::MD_NSCALAR) * sizeof(double), st));
    cgd::FramesDev F = df.dev;
    F.shift = L.shift;
    F.shift_mode = 2;   // the build's images
    mark(ST_SETUP, true);
    cgd::launch_frame_setup(F, df.nghosts, st);
    mark(ST_SETUP, false);
    // The 2-body, 3-body and 4-body parts add into Fo / So with atomics and are
    // otherwise independent: the many-body parts run on two side streams beside the
    // 2-body kernel (a frame of ~1000 atoms gives each contraction only a few warps
    // per SM).  Stage timing keeps them in order on the session stream.
    const bool fork = !profiling_;
    if (fork && !md_side_[0]) {
        for (int k = 0; k < 2; ++k) {
            CK(cudaStreamCreateWithFlags(&md_side_[k], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&md_join_[k], cudaEventDisableTiming));
        }
        CK(cudaEventCreateWithFlags(&md_fork_, cudaEventDisableTiming));
    }
    if (fork) CK(cudaEventRecord(md_fork_, st));
    mark(ST_FORCE2, true);
    cgd::launch_md2(M, D, F, L.NB, Fo, So, st, md_->precision);
    mark(ST_FORCE2, false);
    bool joined[2] = {false, false};
    for (int k = 0; k < 2; ++k) {
        const int64_t n = L.ncl[k];
        if (n == 0 || !L.tstep[k]) continue;
        cudaStream_t sk = fork ? md_side_[k] : st;
        if (fork) CK(cudaStreamWaitEvent(sk, md_fork_, 0));
        cgd::ClusterSet CS = L.CS[k];
        mark(ST_BUCKET, true);
        cgd::launch_md_filter(3 + k, M, F, CS, L.cfo[k], n, L.tstep[k], sk);
        CS.type = L.tstep[k];
        cgd::launch_md_bucket(n, nf, L.cfo[k], L.tstep[k], L.B[k], sk);
        mark(ST_BUCKET, false);
        const int64_t max_tiles = (n + cgd::MDC_TILE - 1) / cgd::MDC_TILE + L.B[k].nkeys;
        mark(k == 0 ? ST_FORCE3 : ST_FORCE4, true);
        cgd::launch_mdc(3 + k, md_->precision, k == 0 ? M.order3 : M.order4, max_tiles, M, D, F, CS, L.B[k], Fo, So,
                        sk);
        mark(k == 0 ? ST_FORCE3 : ST_FORCE4, false);
        if (fork) {
            CK(cudaEventRecord(md_join_[k], sk));
            joined[k] = true;
        }
    }
    for (int k = 0; k < 2; ++k)
        if (joined[k]) CK(cudaStreamWaitEvent(st, md_join_[k], 0));
    if (D.coulomb) {   // ZCalc_Ewald
        const int km = md_ewald_kmax(df);
        void* ews = nullptr;
        CK(cudaMallocAsync(&ews, cgd::md_ewald_scratch_bytes(nf, km), st));
        cgd::launch_md_ewald(nf, nreal, km, M, D, F, ews, Fo, So, st);
        CK(cudaFreeAsync(ews, st));
    }
    cgd::launch_md_finalize(nf, M, D, F, So, st);
    CK(cudaGetLastError());
}

double Session::md_lists_disp2(const DeviceFrames& df, MdLists& L) {
    if (!L.valid || L.natoms != df.natoms_total) return HUGE_VAL;
    cudaStream_t st = stream_;
    CK(cudaMemsetAsync(L.dmax, 0, sizeof(unsigned long long), st));
    cgd::launch_md_maxdisp(df.xyz, L.xref, L.natoms, L.dmax, st);
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, L.dmax, sizeof(bits), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double d2;
    std::memcpy(&d2, &bits, sizeof(d2));
    return d2;
}

void Session::md_force_step(DeviceFrames& df, MdListSet& LS, double* Fo, double* So) {
    if (LS.next_ready) {   // built ahead during the previous step (that build has completed)
        LS.cur ^= 1;
        LS.next_ready = false;
    }
    MdLists& L = LS.current();
    const double half2 = 0.25 * md_skin_ * md_skin_;
    double d2 = md_lists_disp2(df, L);
    if (!(d2 <= half2) || L.skin != md_skin_) {
        md_lists_build(df, md_skin_, L, stream_);
        d2 = 0.0;
    }
    const bool ahead = d2 > (0.75 * 0.75) * half2;   // 3/8 of the skin
    if (ahead) {
        if (!side_stream_) {
            CK(cudaStreamCreateWithFlags(&side_stream_, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&side_event_, cudaEventDisableTiming));
        }
        CK(cudaEventRecord(side_event_, stream_));   // this step's positions
        CK(cudaStreamWaitEvent(side_stream_, side_event_, 0));
    }
    md_force_lists(df, L, Fo, So);
    if (ahead) {   // overlaps the force kernels just queued on the main stream
        md_lists_build(df, md_skin_, LS.lists[LS.cur ^ 1], side_stream_);
        LS.next_ready = true;
        ++LS.early_builds;
    }
}

void Session::subtract_coulomb(FrameBatch& fb) {
    CK(cudaSetDevice(device_));
    const Model& m = model_;
    if (!m.ctl.use_partial_charges) return;
    if (fb.nframes == 0) return;
    if (m.ctl.natmtyp > 10) throw Error(2, "Ewald sums support up to 10 atom types");
    cgd::MdDev D{};
    D.coulomb = 1;
    for (int i = 0; i < m.ctl.natmtyp; ++i) D.qtype[i] = m.pairs[i].chg1;   // ATOM_PAIRS[i].ATM1CHG
    // the first frame's parameters for every frame (static alpha / r_cut / k_cut)
    const cgd::BoxDev& b0 = fb.box[0];
    if (!b0.is_ortho) throw Error(2, "the Ewald sums need an orthorhombic cell");
    Box bx;
    bx.ax = b0.h[0]; bx.by = b0.h[4]; bx.cz = b0.h[8];
    const EwaldParams ep = ewald_params(fb.natoms[0], bx);
    FrameBatch fe = fb;
    for (auto& b : fe.box) {
        if (!b.is_ortho) throw Error(2, "the Ewald sums need an orthorhombic cell");
        b.ew_alpha = ep.alpha; b.ew_rc = ep.rc; b.ew_kmax = ep.kmax;
    }
    std::unique_ptr<DeviceFrames> df = upload(fe);
    cudaStream_t st = stream_;
    const int nf = df->nframes;
    const int64_t n = df->natoms_total;
    Scratch S(st);
    double* Fo = S.get<double>(3 * n);
    double* So = S.get<double>((size_t)nf * cgd::MD_NSCALAR);
    void* ews = S.get<unsigned char>(cgd::md_ewald_scratch_bytes(nf, std::max(1, ep.kmax)));
    CK(cudaMemsetAsync(Fo, 0, sizeof(double) * 3 * n, st));
    CK(cudaMemsetAsync(So, 0, sizeof(double) * nf * cgd::MD_NSCALAR, st));
    cgd::launch_frame_setup(df->dev, df->nghosts, st);
    cgd::launch_md_ewald(nf, (int)n, std::max(1, ep.kmax), dm_->dev, D, df->dev, ews, Fo, So, st);
    CK(cudaGetLastError());
    std::vector<double> f(3 * n);
    CK(cudaMemcpyAsync(f.data(), Fo, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    for (int k = 0; k < fb.nframes; ++k) {   // FORCES -= ACCEL (force rows come first in each frame)
        const int64_t r0 = fb.row_ofs[k], a0 = fb.atom_ofs[k];
        for (int64_t q = 0; q < 3 * (int64_t)fb.natoms[k]; ++q) fb.b[r0 + q] -= f[3 * a0 + q];
    }
}

void Session::md_nve(DeviceFrames& df, const double* mass_type, double dt, int nsteps, double* v, double* Fo,
                     double* So_steps, double* ke_steps) {
    md_run(df, mass_type, dt, nsteps, MdThermostat{}, v, Fo, So_steps, ke_steps, nullptr);
}

void Session::md_numerical(const FrameBatch& fb, bool stress, double* out) {
    CK(cudaSetDevice(device_));
    if (!md_) throw Error(1, "MD coefficients are not set (cg_md_setup)");
    const double eps = 1.0e-4;
    const int nrep = stress ? 12 : 2;   // (t0 >= t1) components x (+, -), or (expand, contract)
    std::vector<Frame> reps;
    std::vector<double> vols;
    reps.reserve((size_t)fb.nframes * nrep);
    for (int k = 0; k < fb.nframes; ++k) {
        const cgd::BoxDev& B = fb.box[k];
        const double* H = B.h;   // columns a, b, c
        const int n = fb.natoms[k];
        const int64_t a0 = fb.atom_ofs[k];
        auto make = [&](const double L[3][3], bool by_factor, double f) {
            Frame r;
            r.natoms = n;
            r.type.assign(fb.type.begin() + a0, fb.type.begin() + a0 + n);
            r.xyz.resize(3 * (size_t)n);
            for (int i = 0; i < n; ++i) {
                const double* x = &fb.xyz[3 * (a0 + i)];
                double* y = &r.xyz[3 * (size_t)i];
                if (by_factor) {   // BOX::SCALE_BY_FACTOR: to cell coordinates, back with f H
                    const double* I = B.inv;
                    const double s0 = I[0] * x[0] + I[1] * x[1] + I[2] * x[2];
                    const double s1 = I[3] * x[0] + I[4] * x[1] + I[5] * x[2];
                    const double s2 = I[6] * x[0] + I[7] * x[1] + I[8] * x[2];
                    for (int q = 0; q < 3; ++q)
                        y[q] = f * H[3 * q] * s0 + f * H[3 * q + 1] * s1 + f * H[3 * q + 2] * s2;
                } else {   // BOX::SCALE_BY_MATRIX: x' = L x
                    for (int q = 0; q < 3; ++q) y[q] = L[q][0] * x[0] + L[q][1] * x[1] + L[q][2] * x[2];
                }
            }
            double cv[3][3] = {{H[0], H[3], H[6]}, {H[1], H[4], H[7]}, {H[2], H[5], H[8]}};   // a, b, c
            double nv[3][3];
            for (int v = 0; v < 3; ++v)
                for (int q = 0; q < 3; ++q)
                    nv[v][q] = by_factor ? cv[v][q] * f : cv[v][0] * L[q][0] + cv[v][1] * L[q][1] + cv[v][2] * L[q][2];
            Box& bx = r.box;
            bx.ax = nv[0][0]; bx.ay = nv[0][1]; bx.az = nv[0][2];
            bx.bx = nv[1][0]; bx.by = nv[1][1]; bx.bz = nv[1][2];
            bx.cx = nv[2][0]; bx.cy = nv[2][1]; bx.cz = nv[2][2];
            bx.update_cell();
            vols.push_back(bx.vol);
            r.force.assign(3 * (size_t)n, 0.0);
            reps.push_back(std::move(r));
        };
        const double I3[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        if (!stress) {
            make(I3, true, 1.0 + eps);
            make(I3, true, 1.0 - eps);
        } else {
            for (int t0 = 0; t0 < 3; ++t0)
                for (int t1 = 0; t1 <= t0; ++t1)
                    for (int sgn = 0; sgn < 2; ++sgn) {
                        double L[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
                        L[t0][t1] += eps;
                        if (sgn) L[t0][t1] -= 2.0 * eps;
                        make(L, false, 1.0);
                    }
        }
    }
    FrameBatch rb = make_batch(model_, reps, 0);
    make_independent(rb);
    std::unique_ptr<DeviceFrames> d = upload(rb);
    const size_t nF = (size_t)rb.natoms_total * 3, nS = (size_t)rb.nframes * cgd::MD_NSCALAR;
    Scratch S(stream_);
    double* dF = S.get<double>(nF + nS);
    md_force(*d, dF, dF + nF, nullptr);
    std::vector<double> so(nS);
    CK(cudaMemcpyAsync(so.data(), dF + nF, nS * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    CK(cudaStreamSynchronize(stream_));
    auto E = [&](int r) { return so[(size_t)r * cgd::MD_NSCALAR]; };
    for (int k = 0; k < fb.nframes; ++k) {
        const int r0 = k * nrep;
        if (!stress) {   // -(U(1-e) - U(1+e)) / (V(1-e) - V(1+e))
            out[k] = -1.0 * (E(r0 + 1) - E(r0)) / (vols[r0 + 1] - vols[r0]);
            continue;
        }
        const double v0 = fb.box[k].vol;
        int r = r0;
        for (int t0 = 0; t0 < 3; ++t0)
            for (int t1 = 0; t1 <= t0; ++t1, r += 2) {
                const double pe1 = E(r) / (2.0 * eps * v0), pe2 = E(r + 1) / (2.0 * eps * v0);
                out[(size_t)k * 9 + t0 * 3 + t1] = pe2 - pe1;
                out[(size_t)k * 9 + t1 * 3 + t0] = pe2 - pe1;
            }
    }
}

std::vector<double> Session::md_restart_fields(int frame) const {
    const int nf = (int)(md_state_.size() / cgd::MD_TH_STRIDE);
    if (frame < 0 || frame >= nf) throw Error(1, "no MD run state for that frame");
    const double* t = &md_state_[(size_t)frame * cgd::MD_TH_STRIDE];
    const double tfs = 48.888;   // src/functions.h:44
    const MdThermostat& th = md_last_th_;
    std::vector<double> r(29, 0.0);
    r[0] = t[cgd::TH_POSIT]; r[1] = t[cgd::TH_ZETA]; r[2] = t[cgd::TH_FORCE]; r[3] = t[cgd::TH_Q];
    r[4] = t[cgd::TH_POSIT0]; r[5] = t[cgd::TH_FORCE0]; r[6] = t[cgd::TH_ZETA0];
    r[7] = t[cgd::TH_BPOS]; r[8] = t[cgd::TH_BVEL]; r[9] = t[cgd::TH_BFORCE]; r[10] = t[cgd::TH_W];
    r[11] = t[cgd::TH_BPOS0]; r[12] = t[cgd::TH_BFORCE0]; r[13] = t[cgd::TH_BVEL0];
    r[14] = t[cgd::TH_SCALE]; r[15] = t[cgd::TH_VOL0]; r[16] = t[cgd::TH_VOL];
    r[17] = 1.0;                                   // BEREND_MU
    r[21] = th.tau_baro_fs / tfs;                  // BEREND_KP
    r[22] = 1.0;                                   // BEREND_ETA
    r[23] = th.tau_fs / tfs;                       // BEREND_TAU
    r[24] = th.tau_fs; r[25] = th.tau_baro_fs;     // TIME, TIME_BARO
    r[26] = t[cgd::TH_NDOF];
    r[27] = t[cgd::TH_VSCALE];
    r[28] = t[cgd::TH_KCUR];
    return r;
}

void Session::md_resume(int nframes, const double* c29) {
    if (nframes < 0 || (nframes > 0 && !c29)) throw Error(1, "resume state arrays");
    md_resume_.assign(c29, c29 + (size_t)nframes * 29);
}

void Session::md_run(DeviceFrames& df, const double* mass_type, double dt, int nsteps, const MdThermostat& th, double* v,
                     double* Fo, double* So_steps, double* ke_steps, double* cons_steps, double* vol_steps) {
    CK(cudaSetDevice(device_));
    if (!md_) throw Error(1, "MD coefficients are not set (cg_md_setup)");
    if (nsteps < 0) throw Error(1, "negative step count");
    const int nt = model_.ctl.natmtyp;
    std::vector<double> m(mass_type, mass_type + nt), im(nt);
    for (int i = 0; i < nt; ++i) {
        if (!(m[i] > 0.0)) throw Error(1, "atom masses must be positive");
        im[i] = 1.0 / m[i];
    }
    cudaStream_t st = stream_;
    const int nf = df.nframes;
    const int64_t n = df.natoms_total;
    Scratch S(st);
    double* dm = S.get<double>(nt);
    double* dim = S.get<double>(nt);
    double* acc = S.get<double>(3 * n);
    double* so = S.get<double>((size_t)nf * cgd::MD_NSCALAR);
    CK(cudaMemcpyAsync(dm, m.data(), nt * sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dim, im.data(), nt * sizeof(double), cudaMemcpyHostToDevice, st));
    const cgd::FramesDev& F = df.dev;
    // thermostat state per frame (CONSTRAINT::INITIALIZE src/ClassDefs.C:525-585):
    // N_DOF = 3N - 3, Q = N_DOF kB T tau^2 / Tfs^2 (tau in fs), Berendsen tau / Tfs
    const double kb = 0.0019872067, tfs = 48.888, gpa = 6.9476955;   // src/functions.h:43-45
    double* thd = nullptr;
    int* bad = nullptr;
    const bool baro = th.style >= 3 && th.style <= 5;
    if (th.style < 0 || th.style > 6) throw Error(1, "unknown thermostat / barostat style");
    const int scale_freq = th.style == 6 ? (int)th.tau_fs : 0;   // NVT-SCALE: steps between rescalings
    if (th.style == 6 && (scale_freq < 1 || (double)scale_freq != th.tau_fs))
        throw Error(1, "NVT-SCALE needs a whole number of steps between rescalings");
    if (baro) {   // src/chimes_md.C:556-563: orthorhombic cells only
        if (!(th.tau_baro_fs > 0.0)) throw Error(1, "the barostat needs a positive time constant");
        for (const auto& b : df.box_host)
            if (!b.is_ortho) throw Error(2, "NPT-BEREND, NPT-BEREND-ANISO and NPT-MTK need orthorhombic cells");
        if (md_->dev.coulomb) throw Error(2, "NPT with Ewald charges is not supported by this library");
    }
    const double p0 = th.pressure_gpa / gpa;
    if (th.style != 0) {
        if (!(th.temperature > 0.0) || !(th.tau_fs > 0.0))
            throw Error(1, "the thermostat needs a positive temperature and time constant");
        std::vector<double> h((size_t)nf * cgd::MD_TH_STRIDE, 0.0);
        for (int f = 0; f < nf; ++f) {
            const double ndof = 3.0 * df.natoms_host.at(f) - 3.0;
            double* t = &h[(size_t)f * cgd::MD_TH_STRIDE];
            t[cgd::TH_Q] = ndof * kb * th.temperature * th.tau_fs * th.tau_fs / tfs / tfs;
            t[cgd::TH_NDOFKT] = ndof * kb * th.temperature;
            t[cgd::TH_W] = (ndof + 3.0) * kb * th.temperature * th.tau_baro_fs * th.tau_baro_fs / tfs / tfs;
            t[cgd::TH_NDOF] = ndof;
            t[cgd::TH_NDOF1KT] = (ndof + 1.0) * kb * th.temperature;
            t[cgd::TH_SCALE] = 1.0;
            t[cgd::TH_VSCALE] = 1.0;
        }
        if (!md_resume_.empty()) {   // CONSTRAINT::READ: the restart file's values
            if (md_resume_.size() != (size_t)nf * 29) throw Error(1, "resume state was given for another frame count");
            for (int f = 0; f < nf; ++f) {
                const double* r = &md_resume_[(size_t)f * 29];
                double* t = &h[(size_t)f * cgd::MD_TH_STRIDE];
                t[cgd::TH_POSIT] = r[0]; t[cgd::TH_ZETA] = r[1]; t[cgd::TH_FORCE] = r[2]; t[cgd::TH_Q] = r[3];
                t[cgd::TH_POSIT0] = r[4]; t[cgd::TH_FORCE0] = r[5]; t[cgd::TH_ZETA0] = r[6];
                t[cgd::TH_BPOS] = r[7]; t[cgd::TH_BVEL] = r[8]; t[cgd::TH_BFORCE] = r[9]; t[cgd::TH_W] = r[10];
                t[cgd::TH_BPOS0] = r[11]; t[cgd::TH_BFORCE0] = r[12]; t[cgd::TH_BVEL0] = r[13];
                t[cgd::TH_SCALE] = r[14]; t[cgd::TH_VOL0] = r[15]; t[cgd::TH_VOL] = r[16];
                t[cgd::TH_VSCALE] = r[27];
            }
        }
        thd = S.get<double>(h.size());
        bad = S.get<int>(1);
        CK(cudaMemcpyAsync(thd, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemsetAsync(bad, 0, sizeof(int), st));
    }
    MdListSet lists;
    cgd::BoxDev* dbox = const_cast<cgd::BoxDev*>(F.box);   // the barostats rescale the cells in place
    const double* so_prev = nullptr;
    for (int step = 0; step <= nsteps; ++step) {
        if (step > 0) {   // UPDATE_COORDS + VELOCS_HALF_1
            if (th.style == 1) cgd::launch_md_mtk_half1(nf, F, dm, df.xyz, v, acc, dt, thd, st);
            else if (th.style == 3 || th.style == 4)
                cgd::launch_md_npt_berend(nf, F, dbox, dm, df.xyz, v, acc, dt, so_prev, p0, th.tau_baro_fs / tfs,
                                          th.style == 4, bad, st);
            else if (th.style == 5) cgd::launch_md_nptmtk_half1(nf, F, dbox, dm, df.xyz, v, acc, dt, thd, st);
            else cgd::launch_md_drift(n, F, nullptr, df.xyz, v, acc, dt, st);
        }
        double* sout = So_steps ? So_steps + (size_t)step * nf * cgd::MD_NSCALAR : so;
        so_prev = sout;
        if (md_skin_ > 0.0 && !baro) {   // a changing cell rebuilds every step
            md_force_step(df, lists, Fo, sout);
        } else {
            md_force(df, Fo, sout, nullptr);
        }
        double* ke = ke_steps ? ke_steps + (size_t)step * nf : nullptr;
        if (th.style == 1 && step > 0) {   // a = F/m, VELOCS_HALF_2 with the MTK iteration
            cgd::launch_md_mtk_half2(nf, F, Fo, dim, dm, acc, v, dt, thd, ke, st);
        } else if (th.style == 5 && step > 0) {   // with the barostat
            cgd::launch_md_nptmtk_half2(nf, F, Fo, dim, dm, sout, p0, acc, v, dt, thd, ke, st);
        } else {
            cgd::launch_md_kick(nf, F, Fo, dim, dm, acc, v, dt, step > 0 ? 1 : 0, nullptr, ke, st);
            if ((th.style == 2 || th.style == 3 || th.style == 4) && step > 0)
                cgd::launch_md_berend(nf, F, dm, v, dt, th.tau_fs / tfs, th.temperature, kb, ke, bad, st);
        }
        if (th.style == 6) cgd::launch_md_vscale(nf, F, dm, v, thd, step, scale_freq, th.temperature, kb, st);
        if (cons_steps && thd) {   // CONSERVED_QUANT (NVT-MTK, NPT-MTK)
            cgd::launch_md_conserved(nf, thd, th.style == 1 ? 1 : (th.style == 5 ? 2 : 0), p0, F.box,
                                     cons_steps + (size_t)step * nf, st);
        }
        if (vol_steps) cgd::launch_md_volume(nf, F.box, vol_steps + (size_t)step * nf, st);
        CK(cudaGetLastError());
    }
    md_resume_.clear();
    md_last_th_ = th;
    md_state_.assign((size_t)nf * cgd::MD_TH_STRIDE, 0.0);
    if (thd) {
        CK(cudaMemcpyAsync(md_state_.data(), thd, md_state_.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    } else {   // NVE: the constraint holds only its degrees of freedom
        for (int f = 0; f < nf; ++f) {
            double* t = &md_state_[(size_t)f * cgd::MD_TH_STRIDE];
            t[cgd::TH_NDOF] = 3.0 * df.natoms_host.at(f) - 3.0;
            t[cgd::TH_SCALE] = 1.0;
            t[cgd::TH_VSCALE] = 1.0;
        }
    }
    CK(cudaStreamSynchronize(st));
    if (baro) {   // keep the host copy of the cells current
        CK(cudaMemcpyAsync(df.box_host.data(), F.box, df.box_host.size() * sizeof(cgd::BoxDev),
                           cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    if (bad) {
        int hb = 0;
        CK(cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hb) throw Error(2, "a Berendsen scale factor became negative: decrease the time step or increase the "
                               "thermostat / barostat time");
    }
}

}  // namespace cg

// ------------------------------------------------------------------ serving loop
namespace cg {
namespace {

// Device bytes of one serving arena (the arrays ServeArena::init allocates).
size_t arena_bytes(int64_t atoms, int frames, int nimg) {
    auto r = [](size_t n, size_t esz) { return std::max<size_t>(n, 1) * esz; };
    return r(frames, 4) + 3 * r(frames + 1, 8) + 2 * r(frames, 4) + r(frames, sizeof(cgd::BoxDev)) + r(atoms, 4) +
           4 * r(3 * atoms, 8) + r((size_t)frames * cgd::MD_NSCALAR, 8) + r(3 * atoms * nimg, 8) +
           r(4 * atoms * nimg, 4) + r(frames, 1);
}

// Device arrays of one batch composition, sized for the largest batch.
struct ServeArena {
    std::vector<void*> allocs;
    int* natoms = nullptr;
    int64_t *atom_ofs = nullptr, *ghost_ofs = nullptr, *row_ofs = nullptr;
    int *stress_rows = nullptr, *energy_rows = nullptr, *type = nullptr;
    cgd::BoxDev* box = nullptr;
    double *xyz = nullptr, *v = nullptr, *acc = nullptr, *scaled = nullptr, *Fo = nullptr, *So = nullptr;
    float* cart32 = nullptr;
    unsigned char* first = nullptr;
    template <typename T>
    T* get(size_t n) {
        void* p = nullptr;
        CK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
        allocs.push_back(p);
        CK(cudaMemset(p, 0, std::max<size_t>(n, 1) * sizeof(T)));
        return reinterpret_cast<T*>(p);
    }
    void init(int64_t atoms, int frames, int nimg) {
        natoms = get<int>(frames);
        atom_ofs = get<int64_t>(frames + 1);
        ghost_ofs = get<int64_t>(frames + 1);
        row_ofs = get<int64_t>(frames + 1);
        stress_rows = get<int>(frames);
        energy_rows = get<int>(frames);
        box = get<cgd::BoxDev>(frames);
        type = get<int>(atoms);
        xyz = get<double>(3 * atoms);
        v = get<double>(3 * atoms);
        acc = get<double>(3 * atoms);
        Fo = get<double>(3 * atoms);
        So = get<double>((size_t)frames * cgd::MD_NSCALAR);
        scaled = get<double>(3 * atoms * nimg);
        cart32 = get<float>(4 * atoms * nimg);
        first = get<unsigned char>(frames);
    }
    ~ServeArena() { for (void* p : allocs) cudaFree(p); }
};

template <typename T>
struct Pinned {
    T* p = nullptr;
    size_t n = 0;
    void reserve(size_t m) {
        if (m <= n) return;
        if (p) cudaFreeHost(p);
        CK(cudaMallocHost((void**)&p, std::max<size_t>(m, 1) * sizeof(T)));
        n = m;
    }
    ~Pinned() { if (p) cudaFreeHost(p); }
};

double now_s(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

void Session::md_serve_memory(int64_t max_batch_atoms, int max_batch_frames, double* arena, double* per_atom) const {
    const int L = model_.ctl.nlayers;
    const int nimg = (2 * L + 1) * (2 * L + 1) * (2 * L + 1);
    if (arena) *arena = 2.0 * (double)arena_bytes(max_batch_atoms, std::max(1, max_batch_frames), nimg);
    if (per_atom) *per_atom = 2.0 * serve_list_per_atom_;
}

cgd::BoxDev Session::serve_check(const MdRequest& q, const MdServeOptions& opt, const std::string& who) const {
    const Model& m = model_;
    const int nt = m.ctl.natmtyp;
    if (q.natoms <= 0 || q.nsteps <= 0 || !q.types || !q.xyz || !q.cell || !q.v)
        throw Error(1, who + ": empty or incomplete");
    if (q.natoms > opt.max_batch_atoms) throw Error(1, who + ": larger than the batch capacity");
    if (q.natoms > 8191) throw Error(2, "frames above 8191 atoms are not supported on the device");
    for (int a = 0; a < q.natoms; ++a)
        if (q.types[a] < 0 || q.types[a] >= nt) throw Error(1, who + ": atom type index out of range");
    Box b;
    b.ax = q.cell[0]; b.ay = q.cell[1]; b.az = q.cell[2]; b.bx = q.cell[3]; b.by = q.cell[4]; b.bz = q.cell[5];
    b.cx = q.cell[6]; b.cy = q.cell[7]; b.cz = q.cell[8];
    b.update_cell();
    if (b.ax <= 0.0 || b.by <= 0.0 || b.cz <= 0.0 || b.ay != 0.0 || b.az != 0.0 || b.bz != 0.0)
        throw Error(2, "cell must be upper triangular with a positive diagonal");
    cgd::BoxDev bd;
    std::memset(&bd, 0, sizeof(bd));
    for (int k = 0; k < 9; ++k) { bd.h[k] = b.hmat[k]; bd.inv[k] = b.invr[k]; }
    bd.lx = b.lx; bd.ly = b.ly; bd.lz = b.lz; bd.vol = b.vol;
    bd.is_ortho = b.is_ortho ? 1 : 0;
    set_small(bd, frame_is_small(m, b, false));
    if (md_ && md_->dev.coulomb) {   // optimal_ewald_params for the request's cell
        if (!b.is_ortho) throw Error(2, "the Ewald sums need an orthorhombic cell");
        const EwaldParams ep = ewald_params(q.natoms, b);
        bd.ew_alpha = ep.alpha; bd.ew_rc = ep.rc; bd.ew_kmax = ep.kmax;
    }
    return bd;
}

double Session::serve_fixed_bytes(const MdServeOptions& opt) const {
    const int L = model_.ctl.nlayers;
    const int nimg = (2 * L + 1) * (2 * L + 1) * (2 * L + 1);
    return 2.0 * (double)arena_bytes(opt.max_batch_atoms, std::max(1, opt.max_batch_frames), nimg);
}

namespace {
// cg_md_serve's requests: a fixed list, offered in order of arrival time.
struct ListSource : ServeSource {
    const std::vector<MdRequest>& req;
    MdResult* res;
    std::vector<int> order;
    size_t next_pending = 0;
    ListSource(const std::vector<MdRequest>& r, MdResult* out) : req(r), res(out), order(r.size()) {
        for (size_t k = 0; k < r.size(); ++k) order[k] = (int)k;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return req[a].arrival < req[b].arrival; });
    }
    int next(double now) override {
        if (next_pending < order.size() && req[order[next_pending]].arrival <= now) return order[next_pending];
        return -1;
    }
    void admitted() override { ++next_pending; }
    const MdRequest& request(int id) override { return req[id]; }
    bool wait(double now) override {
        if (next_pending >= order.size()) return false;
        const double w = req[order[next_pending]].arrival - now;
        if (w > 0) std::this_thread::sleep_for(std::chrono::duration<double>(w));
        return true;
    }
    void finished(int id, const MdResult& r) override { res[id] = r; }
};
}  // namespace

int64_t Session::md_serve(const std::vector<MdRequest>& req, const double* mass_type, const MdServeOptions& opt,
                          MdResult* res, double* step_ms) {
    CK(cudaSetDevice(device_));
    if (!md_) throw Error(1, "MD coefficients are not set (cg_md_setup)");
    const double fixed = serve_fixed_bytes(opt);
    if (fixed > opt.hbm_budget)
        throw Error(1, "hbm_budget of " + std::to_string((long long)opt.hbm_budget) + " bytes is below the " +
                           std::to_string((long long)fixed) + " bytes of the serving arenas for max_batch_atoms");
    int stride = 0;
    for (size_t r = 0; r < req.size(); ++r) {
        serve_check(req[r], opt, "request " + std::to_string(r));
        stride = std::max(stride, req[r].nsteps);
        if (fixed + serve_need_bytes(req[r].natoms) > opt.hbm_budget)
            throw Error(1, "request " + std::to_string(r) + " alone needs more device memory (" +
                               std::to_string((long long)(fixed + serve_need_bytes(req[r].natoms))) +
                               " bytes with the arenas) than hbm_budget allows");
    }
    ListSource src(req, res);
    return serve_loop(src, mass_type, opt, step_ms, stride);
}

int64_t Session::serve_loop(ServeSource& src, const double* mass_type, const MdServeOptions& opt, double* step_ms,
                            int stride) {
    CK(cudaSetDevice(device_));
    if (!md_) throw Error(1, "MD coefficients are not set (cg_md_setup)");
    const Model& m = model_;
    const int nt = m.ctl.natmtyp;
    const int L = m.ctl.nlayers;
    const int nimg = (2 * L + 1) * (2 * L + 1) * (2 * L + 1);
    std::vector<double> mv(mass_type, mass_type + nt), im(nt);
    for (int i = 0; i < nt; ++i) {
        if (!(mv[i] > 0.0)) throw Error(1, "atom masses must be positive");
        im[i] = 1.0 / mv[i];
    }
    cudaStream_t st = stream_;
    const int64_t cap_atoms = opt.max_batch_atoms;
    const int cap_frames = std::max(1, opt.max_batch_frames);
    // Device memory: the two arenas (fixed, allocated below) plus the neighbour /
    // cluster lists of the running composition, which grow with its atoms.  A request
    // of n atoms reserves 2 * list_per_atom * n bytes (the current lists and the set
    // built ahead of need); list_per_atom starts from a prior and is replaced by the
    // lists' measured allocation per atom after every build (never shrinking).
    const double fixed = serve_fixed_bytes(opt);
    if (fixed > opt.hbm_budget)
        throw Error(1, "hbm_budget of " + std::to_string((long long)opt.hbm_budget) + " bytes is below the " +
                           std::to_string((long long)fixed) + " bytes of the serving arenas for max_batch_atoms");
    ServeArena arena[2];
    arena[0].init(cap_atoms, cap_frames, nimg);
    arena[1].init(cap_atoms, cap_frames, nimg);
    double *dm = nullptr, *dim = nullptr;
    CK(cudaMalloc((void**)&dm, nt * sizeof(double)));
    CK(cudaMalloc((void**)&dim, nt * sizeof(double)));
    std::unique_ptr<double, void (*)(double*)> g1(dm, [](double* p) { cudaFree(p); });
    std::unique_ptr<double, void (*)(double*)> g2(dim, [](double* p) { cudaFree(p); });
    CK(cudaMemcpy(dm, mv.data(), nt * sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dim, im.data(), nt * sizeof(double), cudaMemcpyHostToDevice));
    Pinned<int> h_nat, h_type;
    Pinned<int64_t> h_aofs, h_gofs;
    Pinned<cgd::BoxDev> h_box;
    Pinned<unsigned char> h_first;
    h_nat.reserve(cap_frames); h_aofs.reserve(cap_frames + 1); h_gofs.reserve(cap_frames + 1);
    h_box.reserve(cap_frames); h_first.reserve(cap_frames); h_type.reserve(cap_atoms);

    // per-request state, by id
    std::vector<int> steps_done;
    std::vector<int64_t> pos;      // atom offset of each active request in the current arena
    std::vector<char> first;
    std::vector<MdResult> res;
    std::vector<cgd::BoxDev> boxes;
    auto grow = [&](int id) {
        if ((int)steps_done.size() > id) return;
        const size_t n = (size_t)id + 1;
        steps_done.resize(n, 0); pos.resize(n, -1); first.resize(n, 0); res.resize(n); boxes.resize(n);
    };
    std::vector<int> active, done_now;
    int cur = 0;
    int64_t active_atoms = 0, nbatch = 0;
    MdListSet lists;   // skin lists of the current composition
    int64_t builds_seen = 0;
    bool changed = false;
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        // admit every arrived request that fits
        const double t = now_s(t0);
        for (int id; (id = src.next(t)) >= 0;) {
            const MdRequest& q = src.request(id);
            if (active_atoms + q.natoms > cap_atoms || (int)active.size() >= cap_frames) break;
            if (fixed + serve_need_bytes(active_atoms + q.natoms) > opt.hbm_budget) {
                if (active.empty())   // the measured list size leaves no room for it even alone
                    throw Error(4, "request " + std::to_string(id) +
                                       " needs more device memory than hbm_budget allows (measured list size " +
                                       std::to_string((long long)serve_list_per_atom_) + " bytes per atom)");
                break;
            }
            grow(id);
            boxes[id] = serve_check(q, opt, "request " + std::to_string(id));
            src.admitted();
            active.push_back(id);
            active_atoms += q.natoms;
            first[id] = 1;
            res[id].admitted = t;
            res[id].reserved_bytes = serve_need_bytes(q.natoms);
            changed = true;
        }
        if (active.empty()) {
            if (!src.wait(now_s(t0))) break;
            continue;
        }
        ServeArena& A = arena[cur];
        ServeArena& B = arena[cur ^ 1];
        const int nf = (int)active.size();
        if (changed) {
            // new composition in the other arena: carried-over state copied on the device
            int64_t ofs = 0;
            h_aofs.p[0] = 0; h_gofs.p[0] = 0;
            for (int k = 0; k < nf; ++k) {
                const int r = active[k];
                const MdRequest& q = src.request(r);
                const int n = q.natoms;
                h_nat.p[k] = n;
                h_box.p[k] = boxes[r];
                std::memcpy(h_type.p + ofs, q.types, n * sizeof(int));
                if (first[r]) {
                    CK(cudaMemcpyAsync(B.xyz + 3 * ofs, q.xyz, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
                    CK(cudaMemcpyAsync(B.v + 3 * ofs, q.v, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
                    CK(cudaMemsetAsync(B.acc + 3 * ofs, 0, 3 * n * sizeof(double), st));
                } else {
                    const size_t bytes = 3 * n * sizeof(double);
                    CK(cudaMemcpyAsync(B.xyz + 3 * ofs, A.xyz + 3 * pos[r], bytes, cudaMemcpyDeviceToDevice, st));
                    CK(cudaMemcpyAsync(B.v + 3 * ofs, A.v + 3 * pos[r], bytes, cudaMemcpyDeviceToDevice, st));
                    CK(cudaMemcpyAsync(B.acc + 3 * ofs, A.acc + 3 * pos[r], bytes, cudaMemcpyDeviceToDevice, st));
                }
                ofs += n;
                h_aofs.p[k + 1] = ofs;
                h_gofs.p[k + 1] = ofs * nimg;
            }
            for (int k = 0; k < nf; ++k) pos[active[k]] = h_aofs.p[k];
            CK(cudaMemcpyAsync(B.natoms, h_nat.p, nf * sizeof(int), cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(B.atom_ofs, h_aofs.p, (nf + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(B.ghost_ofs, h_gofs.p, (nf + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(B.box, h_box.p, nf * sizeof(cgd::BoxDev), cudaMemcpyHostToDevice, st));
            CK(cudaMemcpyAsync(B.type, h_type.p, ofs * sizeof(int), cudaMemcpyHostToDevice, st));
            cur ^= 1;
            changed = false;
            lists.release();
        }
        ServeArena& C = arena[cur];
        for (int k = 0; k < nf; ++k) h_first.p[k] = first[active[k]] ? 1 : 0;
        CK(cudaMemcpyAsync(C.first, h_first.p, nf, cudaMemcpyHostToDevice, st));
        DeviceFrames df;
        df.nframes = nf;
        df.box_host.assign(h_box.p, h_box.p + nf);
        df.natoms_total = active_atoms;
        df.nghosts = active_atoms * nimg;
        df.xyz = C.xyz;
        cgd::FramesDev& F = df.dev;
        F.nframes = nf; F.nlayers = L; F.nimg = nimg;
        F.natoms = C.natoms; F.atom_ofs = C.atom_ofs; F.ghost_ofs = C.ghost_ofs; F.row_ofs = C.row_ofs;
        F.stress_rows = C.stress_rows; F.energy_rows = C.energy_rows; F.box = C.box; F.type = C.type;
        F.xyz = C.xyz; F.scaled = C.scaled; F.cart32 = C.cart32;
        // one batched step
        const auto s0 = std::chrono::steady_clock::now();
        cgd::launch_md_drift(active_atoms, F, C.first, C.xyz, C.v, C.acc, opt.dt, st);
        if (md_skin_ > 0.0) {
            md_force_step(df, lists, C.Fo, C.So);
        } else {
            md_force(df, C.Fo, C.So, nullptr);
        }
        cgd::launch_md_kick(nf, F, C.Fo, dim, dm, C.acc, C.v, opt.dt, 1, C.first, nullptr, st);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - s0).count();
        ++nbatch;
        // list bytes per atom measured on the lists just built (grow-only buffers)
        const int64_t nbuilds = lists.lists[0].builds + lists.lists[1].builds;
        if (nbuilds != builds_seen && active_atoms > 0) {
            builds_seen = nbuilds;
            size_t bytes = 0;
            for (size_t c : lists.current().caps) bytes += c;
            serve_list_per_atom_ = std::max((double)serve_list_per_atom_, (double)bytes / (double)active_atoms);
        }
        // bookkeeping, retire finished requests
        std::vector<int> keep;
        keep.reserve(active.size());
        done_now.clear();
        for (int r : active) {
            const MdRequest& q = src.request(r);
            if (step_ms && steps_done[r] < stride) step_ms[(size_t)r * stride + steps_done[r]] = ms;
            res[r].step_ms_sum += ms;
            res[r].step_ms_max = std::max(res[r].step_ms_max, ms);
            first[r] = 0;
            if (++steps_done[r] == q.nsteps) {
                if (q.xyz_out)
                    CK(cudaMemcpyAsync(q.xyz_out, C.xyz + 3 * pos[r], 3 * q.natoms * sizeof(double),
                                       cudaMemcpyDeviceToHost, st));
                active_atoms -= q.natoms;
                done_now.push_back(r);
                changed = true;
            } else {
                keep.push_back(r);
            }
        }
        if (!done_now.empty()) {
            CK(cudaStreamSynchronize(st));
            const double tf = now_s(t0);
            for (int r : done_now) {
                res[r].finished = tf;
                src.finished(r, res[r]);
            }
        }
        active.swap(keep);
    }
    return nbatch;
}

// ---------------------------------------------------------------- live serving
MdServer::MdServer(Session& s, const double* mass_type, const MdServeOptions& opt)
    : s_(s), mass_(mass_type, mass_type + s.model().ctl.natmtyp), opt_(opt) {
    const double fixed = s_.serve_fixed_bytes(opt_);
    if (fixed > opt_.hbm_budget)
        throw Error(1, "hbm_budget of " + std::to_string((long long)opt_.hbm_budget) + " bytes is below the " +
                           std::to_string((long long)fixed) + " bytes of the serving arenas for max_batch_atoms");
    for (double mv : mass_)
        if (!(mv > 0.0)) throw Error(1, "atom masses must be positive");
    th_ = std::thread([this] { run(); });
}

MdServer::~MdServer() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stopping_ = true;
    }
    cv_.notify_all();
    if (th_.joinable()) th_.join();
}

void MdServer::run() {
    int code = 0;
    std::string msg;
    int64_t steps = 0;
    try {
        steps = s_.serve_loop(*this, mass_.data(), opt_, nullptr, 0);
    } catch (const Error& e) {
        code = e.code;
        msg = e.what();
    } catch (const std::bad_alloc&) {
        code = 4;
        msg = "out of host memory";
    } catch (const std::exception& e) {
        code = 3;
        msg = e.what();
    }
    std::lock_guard<std::mutex> lk(mu_);
    steps_ = steps;
    err_code_ = code;
    err_msg_ = msg;
    ended_ = true;
    cv_.notify_all();
}

int64_t MdServer::submit(const MdRequest& q) {
    const double fixed = s_.serve_fixed_bytes(opt_);
    s_.serve_check(q, opt_, "request");
    if (fixed + s_.serve_need_bytes(q.natoms) > opt_.hbm_budget)
        throw Error(1, "the request alone needs more device memory (" +
                           std::to_string((long long)(fixed + s_.serve_need_bytes(q.natoms))) +
                           " bytes with the arenas) than hbm_budget allows");
    std::unique_lock<std::mutex> lk(mu_);
    if (stopping_ || ended_) throw Error(1, "the server has stopped");
    t_.emplace_back();
    Ticket& k = t_.back();
    k.types.assign(q.types, q.types + q.natoms);
    k.xyz.assign(q.xyz, q.xyz + 3 * (size_t)q.natoms);
    k.cell.assign(q.cell, q.cell + 9);
    k.v.assign(q.v, q.v + 3 * (size_t)q.natoms);
    k.out.assign(3 * (size_t)q.natoms, 0.0);
    k.q.natoms = q.natoms;
    k.q.nsteps = q.nsteps;
    k.q.arrival = 0.0;
    k.q.types = k.types.data();
    k.q.xyz = k.xyz.data();
    k.q.cell = k.cell.data();
    k.q.v = k.v.data();
    k.q.xyz_out = k.out.data();
    const int64_t ticket = (int64_t)t_.size() - 1;
    lk.unlock();
    cv_.notify_all();
    return ticket;
}

int MdServer::poll(int64_t ticket, bool wait, MdResult* r, double* xyz) {
    std::unique_lock<std::mutex> lk(mu_);
    if (ticket < 0 || ticket >= (int64_t)t_.size()) throw Error(1, "unknown ticket");
    Ticket& k = t_[(size_t)ticket];
    if (wait) cv_.wait(lk, [&] { return k.done || ended_; });
    if (k.done) {
        if (r) *r = k.res;
        if (xyz) std::memcpy(xyz, k.out.data(), k.out.size() * sizeof(double));
        return 0;
    }
    if (ended_) {
        if (err_code_) throw Error(err_code_, "serving loop failed: " + err_msg_);
        throw Error(1, "the server stopped before this request finished");
    }
    return CG_PENDING_STATUS;
}

int64_t MdServer::stop() {
    {
        std::lock_guard<std::mutex> lk(mu_);
        stopping_ = true;
    }
    cv_.notify_all();
    if (th_.joinable()) th_.join();
    if (err_code_) throw Error(err_code_, "serving loop failed: " + err_msg_);
    return steps_;
}

int MdServer::next(double) {
    std::lock_guard<std::mutex> lk(mu_);
    return next_ < t_.size() ? (int)next_ : -1;
}

void MdServer::admitted() {
    std::lock_guard<std::mutex> lk(mu_);
    ++next_;
}

const MdRequest& MdServer::request(int id) {
    std::lock_guard<std::mutex> lk(mu_);
    return t_[(size_t)id].q;   // deque elements do not move when the queue grows
}

bool MdServer::wait(double) {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] { return next_ < t_.size() || stopping_; });
    return next_ < t_.size();
}

void MdServer::finished(int id, const MdResult& r) {
    {
        std::lock_guard<std::mutex> lk(mu_);
        t_[(size_t)id].res = r;
        t_[(size_t)id].done = true;
    }
    cv_.notify_all();
}

}  // namespace cg
