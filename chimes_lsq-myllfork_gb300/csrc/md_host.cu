// Host orchestration of the MD force and the NVE integrator on one GPU.
//
//   ZCalc             src/functions.C:815-891   -> Session::md_force
//   chimes_md MD loop src/chimes_md.C:700-1050  -> Session::md_nve (NVE only)
//
// The per-step launch sequence is the design-matrix path's enumeration (ghosts,
// neighbour lists, clusters, per-(frame, type) buckets) followed by the force
// kernels of md.cu.
#include <algorithm>
#include <cmath>
#include <vector>

#include "assemble.h"
#include "kernels.h"
#include "md.h"
#include "scratch.h"
#include "session.h"

namespace cg {

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
    // 2-body: x[pt * order2 + n] multiplies T_{n+1} (src/chimes_lsq.py:462-477 layout)
    std::vector<double> c2((size_t)m.pairs.size() * o2);
    for (size_t i = 0; i < c2.size(); ++i) c2[i] = x[i];
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
    if (offsets) {
        if (m.tot_all - m.tot_short != m.ctl.natmtyp) throw Error(2, "the model has no energy-offset columns");
        t->dev.eoff = (const double*)up(x + m.tot_short, m.ctl.natmtyp * sizeof(double));
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
    CK(cudaStreamSynchronize(st));
    NB.i2 = S.get<int>(tot[0]); NB.g2 = S.get<int>(tot[0]); NB.pt2 = S.get<int>(tot[0]);
    NB.r2 = S.get<double>(tot[0]); NB.rab2 = S.get<double>(3 * tot[0]);
    NB.g3 = S.get<int>(tot[1]); NB.r3 = S.get<double>(tot[1]);
    NB.g4 = S.get<int>(tot[2]); NB.r4 = S.get<double>(tot[2]);
    cgd::launch_neigh(M, F, NB, 1, st); L();
    c.pairs2 = tot[0];
    cgd::launch_md2(M, D, F, NB, Fo, So, st); L();
    CK(cudaGetLastError());
    int64_t* kfo_atoms = S.get<int64_t>(nf + 1);
    cgd::launch_key_frame_ofs(F.atom_ofs, nf, 0, kfo_atoms, st); L();
    auto many = [&](int nbody, int ntypes, int ord) {
        cgd::ClusterSet CS{};
        CS.cnt = S.get<int>(nreal);
        CS.ofs = S.get<int64_t>(nreal + 1);
        cgd::launch_clusters(nbody, M, F, NB, CS, 0, st); L();
        cgd::launch_scan_counts(CS.cnt, nreal, CS.ofs, st); L();
        int64_t n = 0;
        CK(cudaMemcpyAsync(&n, CS.ofs + nreal, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        (nbody == 3 ? c.triplets : c.quads) = n;
        if (n == 0) return;
        CS.m = S.get<int4>(n);
        CS.type = S.get<int>(n);
        cgd::launch_clusters(nbody, M, F, NB, CS, 1, st); L();
        int64_t* cfo = S.get<int64_t>(nf + 1);
        cgd::launch_gather_frame_ofs(CS.ofs, F.atom_ofs, nf, cfo, st); L();
        int64_t* kfo = S.get<int64_t>(nf + 1);
        cgd::launch_key_frame_ofs(F.atom_ofs, nf, ntypes, kfo, st); L();
        cgd::Buckets byt{S.get<int64_t>((int64_t)nf * (ntypes + 1)), S.get<int>(n)};
        cgd::BucketSpec spec{2, 1, cfo, kfo, nullptr, nullptr, nullptr, CS.type};
        cgd::launch_bucket(nf, F, spec, byt, st); L();
        int* dmax = S.get<int>(1);
        CK(cudaMemsetAsync(dmax, 0, sizeof(int), st));
        cgd::launch_max_bucket(byt.key_ofs, kfo, nf, ntypes, dmax, st); L();
        int hmax = 0;
        CK(cudaMemcpyAsync(&hmax, dmax, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        cgd::launch_mdc(nbody, md_->precision, nf, ntypes, ord, hmax, M, D, F, CS, byt, kfo, Fo, So, st); L();
        CK(cudaGetLastError());
    };
    if (M.order3 > 0) many(3, M.ntypes3, M.order3);
    if (M.order4 > 0) many(4, M.ntypes4, M.order4);
    cgd::launch_md_finalize(nf, M, D, F, So, st); L();
    CK(cudaGetLastError());
    if (counts) *counts = c;
}

void Session::md_nve(DeviceFrames& df, const double* mass_type, double dt, int nsteps, double* v, double* Fo,
                     double* So_steps, double* ke_steps) {
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
    for (int step = 0; step <= nsteps; ++step) {
        if (step > 0) cgd::launch_md_drift(n, df.xyz, v, acc, dt, st);   // UPDATE_COORDS + VELOCS_HALF_1
        double* sout = So_steps ? So_steps + (size_t)step * nf * cgd::MD_NSCALAR : so;
        md_force(df, Fo, sout, nullptr);
        cgd::launch_md_kick(nf, F, Fo, dim, dm, acc, v, dt, step > 0 ? 1 : 0,
                            ke_steps ? ke_steps + (size_t)step * nf : nullptr, st);   // a = F/m, VELOCS_HALF_2
        CK(cudaGetLastError());
    }
}

}  // namespace cg
