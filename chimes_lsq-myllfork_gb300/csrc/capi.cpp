// extern "C" entry points declared in include/chimes_gb300.h.
#include "../../include/chimes_gb300.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "model.h"
#include "session.h"
#include "md_server.h"
#include "textio.h"
#include "mdio.h"

struct cg_model {
    cg::Model m;
};
struct cg_frames {
    cg::FrameBatch fb;
};
struct cg_session {
    std::unique_ptr<cg::Session> s;
    cg::AssembleStats last;
    cg::MdCounts md_last;
};
struct cg_md_server {
    std::unique_ptr<cg::MdServer> srv;
};
struct cg_batch_fit {
    std::unique_ptr<cg::BatchFit> b;
};
struct cg_dframes {
    std::unique_ptr<cg::DeviceFrames> d;
    int64_t nrows = 0;
};

static thread_local std::string g_err;

template <typename F>
static int guarded(F&& fn) {
    try {
        g_err.clear();
        fn();
        return 0;
    } catch (const cg::Error& e) {
        g_err = e.what();
        return e.code;
    } catch (const std::bad_alloc&) {
        g_err = "out of host memory";
        return 4;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 2;
    }
}

static void need(bool ok, const char* what) {
    if (!ok) throw cg::Error(1, std::string("bad argument: ") + what);
}

extern "C" {

const char* cg_last_error(void) { return g_err.c_str(); }

int cg_model_load(const char* path, cg_model** out) {
    return guarded([&] {
        need(path && out, "path/out");
        std::unique_ptr<cg_model> h(new cg_model());
        h->m = cg::load_model(path);
        *out = h.release();
    });
}

void cg_model_free(cg_model* m) { delete m; }

int cg_model_columns(const cg_model* h, int* n2b, int* n3b, int* n4b, int* nener, int* ntotal) {
    return guarded([&] {
        need(h, "model");
        if (n2b) *n2b = h->m.tot_snum;
        if (n3b) *n3b = h->m.num3;
        if (n4b) *n4b = h->m.num4;
        if (nener) *nener = h->m.tot_all - h->m.tot_short - h->m.ncoul;
        if (ntotal) *ntotal = h->m.tot_all;
    });
}

int cg_model_charge_columns(const cg_model* h, int* ncoul, int* nconstraints) {
    return guarded([&] {
        need(h, "model");
        if (ncoul) *ncoul = h->m.ncoul;
        if (nconstraints) *nconstraints = (int)h->m.charge_constraints.size();
    });
}

int cg_model_constraint_rows(const cg_model* h, double* A, int64_t lda, double* b) {
    return guarded([&] {
        need(h && (h->m.charge_constraints.empty() || (A && b)), "model/A/b");
        need(lda >= h->m.tot_all, "lda");
        cg::constraint_rows(h->m, A, lda, b);
    });
}

int cg_model_row_layout(const cg_model* h, int* stress_rows, int* energy_rows) {
    return guarded([&] {
        need(h, "model");
        const cg::Controls& c = h->m.ctl;
        if (stress_rows) *stress_rows = c.fit_stress_all ? 9 : (c.fit_stress ? 3 : 0);
        if (energy_rows) *energy_rows = c.fit_ener ? 3 : 0;
    });
}

int cg_model_sizes(const cg_model* h, int* nframes, int* natmtyp) {
    return guarded([&] {
        need(h, "model");
        if (nframes) *nframes = h->m.ctl.nframes;
        if (natmtyp) *natmtyp = h->m.ctl.natmtyp;
    });
}

static void copy_text(const std::string& t, char* buf, size_t cap, size_t* needed) {
    if (needed) *needed = t.size();
    if (buf && cap) {
        size_t n = t.size() < cap - 1 ? t.size() : cap - 1;
        std::memcpy(buf, t.data(), n);
        buf[n] = 0;
    }
}

int cg_model_header_text(const cg_model* h, char* buf, size_t cap, size_t* needed) {
    return guarded([&] {
        need(h, "model");
        copy_text(cg::params_header_text(h->m), buf, cap, needed);
    });
}

int cg_model_map_text(const cg_model* h, char* buf, size_t cap, size_t* needed) {
    return guarded([&] {
        need(h, "model");
        copy_text(cg::ff_groups_map_text(h->m), buf, cap, needed);
    });
}

int cg_model_params_text(const cg_model* h, const double* x, int nx, const char* preamble, char* buf, size_t cap,
                         size_t* needed) {
    return guarded([&] {
        need(h && x, "model/x");
        copy_text(cg::params_txt_text(h->m, x, nx, preamble ? preamble : ""), buf, cap, needed);
    });
}

int cg_model_params_read(const cg_model* h, const char* text, double* x, int nx) {
    return guarded([&] {
        need(h && text && x, "model/text/x");
        need(nx == h->m.tot_all, "coefficient count");
        std::vector<double> v = cg::params_txt_coefficients(h->m, text);
        std::copy(v.begin(), v.end(), x);
    });
}

int cg_frames_read(const cg_model* h, const char* path, int nframes, cg_frames** out) {
    return guarded([&] {
        need(h && out, "model/out");
        std::vector<cg::Frame> frames;
        if (!path && nframes <= 0) {
            frames = cg::read_frames(h->m, 1);
        } else {
            std::string p = path ? std::string(path) : h->m.ctl.infile.at(0);
            if (!path && !p.empty() && p[0] != '/') p = h->m.dir + "/" + p;
            cg::Box box;
            frames = cg::read_xyzf(h->m, p, nframes > 0 ? nframes : h->m.ctl.nframes, 0, box);
        }
        std::unique_ptr<cg_frames> f(new cg_frames());
        f->fb = cg::make_batch(h->m, frames, 0);
        *out = f.release();
    });
}

int cg_frames_read_ranks(const cg_model* h, int nprocs, cg_frames** out) {
    return guarded([&] {
        need(h && out && nprocs >= 1, "model/out/nprocs");
        std::vector<cg::Frame> frames = cg::read_frames(h->m, nprocs);
        std::unique_ptr<cg_frames> f(new cg_frames());
        f->fb = cg::make_batch(h->m, frames, 0, nprocs);
        *out = f.release();
    });
}

int cg_frames_create(const cg_model* h, int nframes, const int* natoms, const int* types, const double* xyz,
                     const double* forces, const double* cell, const double* stress, const double* energy,
                     int first_index, cg_frames** out) {
    return guarded([&] {
        need(h && out && nframes >= 0 && natoms && types && xyz && cell, "frame arrays");
        const double fconv = 627.50960803 * 1.889725989;
        std::vector<cg::Frame> frames(nframes);
        int64_t a0 = 0;
        for (int f = 0; f < nframes; ++f) {
            cg::Frame& fr = frames[f];
            fr.natoms = natoms[f];
            need(fr.natoms > 0, "natoms");
            fr.type.assign(types + a0, types + a0 + fr.natoms);
            for (int t : fr.type) need(t >= 0 && t < h->m.ctl.natmtyp, "atom type index");
            fr.xyz.assign(xyz + 3 * a0, xyz + 3 * (a0 + fr.natoms));
            fr.force.assign(3 * (size_t)fr.natoms, 0.0);
            if (forces)
                for (int k = 0; k < 3 * fr.natoms; ++k) fr.force[k] = forces[3 * a0 + k] * fconv;
            const double* c = cell + 9 * (size_t)f;
            cg::Box& b = fr.box;
            b.ax = c[0]; b.ay = c[1]; b.az = c[2]; b.bx = c[3]; b.by = c[4]; b.bz = c[5];
            b.cx = c[6]; b.cy = c[7]; b.cz = c[8];
            b.update_cell();
            if (b.ax <= 0.0 || b.by <= 0.0 || b.cz <= 0.0 || b.ay != 0.0 || b.az != 0.0 || b.bz != 0.0)
                throw cg::Error(2, "cell must be upper triangular with a positive diagonal");
            if (stress) {
                for (int k = 0; k < 3; ++k) fr.stress_diag[k] = stress[6 * (size_t)f + k];
                for (int k = 0; k < 3; ++k) fr.stress_off[k] = stress[6 * (size_t)f + 3 + k];
            }
            fr.energy = energy ? energy[f] : 0.0;
            a0 += fr.natoms;
        }
        std::unique_ptr<cg_frames> fo(new cg_frames());
        fo->fb = cg::make_batch(h->m, frames, first_index);
        *out = fo.release();
    });
}

void cg_frames_free(cg_frames* fr) { delete fr; }

int cg_frames_rows(const cg_frames* fr, int64_t* nrows, int64_t* natoms) {
    return guarded([&] {
        need(fr, "frames");
        if (nrows) *nrows = fr->fb.nrows;
        if (natoms) *natoms = fr->fb.natoms_total;
    });
}

int cg_write_lsq_files(const cg_model* h, const cg_frames* fr, const double* A, int64_t lda, const char* dir) {
    return guarded([&] {
        need(h && fr && dir, "model/frames/dir");
        need(!A || lda >= h->m.tot_all, "lda");
        cg::write_lsq_files(h->m, fr->fb, A, lda, dir);
    });
}

int cg_frames_independent(cg_frames* fr) {
    return guarded([&] {
        need(fr, "frames");
        cg::make_independent(fr->fb);
    });
}

int cg_frames_slice(const cg_frames* fr, int first, int count, cg_frames** out) {
    return guarded([&] {
        need(fr && out, "frames/out");
        std::unique_ptr<cg_frames> o(new cg_frames());
        o->fb = cg::slice_batch(fr->fb, first, count);
        *out = o.release();
    });
}

int cg_frames_count(const cg_frames* fr, int* nframes) {
    return guarded([&] {
        need(fr && nframes, "frames/nframes");
        *nframes = fr->fb.nframes;
    });
}

int cg_frames_labels(const cg_frames* fr, double* b) {
    return guarded([&] {
        need(fr && b, "frames/b");
        std::memcpy(b, fr->fb.b.data(), fr->fb.b.size() * sizeof(double));
    });
}

int cg_session_create(const cg_model* h, int device, cg_session** out) {
    return guarded([&] {
        need(h && out, "model/out");
        std::unique_ptr<cg_session> s(new cg_session());
        s->s.reset(new cg::Session(h->m, device));
        *out = s.release();
    });
}

void cg_session_free(cg_session* s) { delete s; }

void* cg_session_stream(cg_session* s) { return s ? (void*)s->s->stream() : nullptr; }

int cg_frames_upload(cg_session* s, const cg_frames* fr, cg_dframes** out) {
    return guarded([&] {
        need(s && fr && out, "session/frames/out");
        std::unique_ptr<cg_dframes> d(new cg_dframes());
        d->d = s->s->upload(fr->fb);
        d->nrows = fr->fb.nrows;
        *out = d.release();
    });
}

void cg_dframes_free(cg_dframes* d) { delete d; }

int cg_assemble_device(cg_session* s, const cg_dframes* d, int precision, void* A, int64_t lda) {
    return guarded([&] {
        need(s && d && A, "session/frames/A");
        need(precision == CG_FP64 || precision == CG_FP32, "precision");
        s->s->assemble(*d->d, precision, A, lda, &s->last);
    });
}

int cg_assemble_device_noalloc(cg_session* s, const cg_dframes* d, int precision, void* A, int64_t lda) {
    return guarded([&] {
        need(s && d && A, "session/frames/A");
        need(precision == CG_FP64 || precision == CG_FP32, "precision");
        s->s->assemble_noalloc(*d->d, precision, A, lda, &s->last);
    });
}

// Frames per block of a streamed assembly: about 8 GiB of A per block (smaller
// blocks lose device efficiency to per-block list sizing), at most an eighth of the
// device's free memory (two blocks are resident), at least one frame, and at least
// two blocks when the batch has two frames (so copies overlap).
static int auto_block_frames(int device, const cg::FrameBatch& fb, int64_t lda, size_t rsz) {
    if (fb.nframes <= 1) return 1;
    size_t free_b = 0, total_b = 0;
    cudaSetDevice(device);
    double target = double(size_t(8) << 30);
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) target = std::min(target, (double)free_b / 8.0);
    const double bytes_per_frame = (double)fb.nrows / fb.nframes * (double)lda * (double)rsz;
    int bf = (int)std::max(1.0, target / std::max(1.0, bytes_per_frame));
    return std::max(1, std::min(bf, (fb.nframes + 1) / 2));
}

int cg_assemble(cg_session* s, const cg_frames* fr, int precision, void* A, int64_t lda) {
    return guarded([&] {
        need(s && fr && A, "session/frames/A");
        need(precision == CG_FP64 || precision == CG_FP32, "precision");
        const size_t rsz = precision == CG_FP64 ? 8 : 4;
        char* base = static_cast<char*>(A);
        s->s->assemble_to_host(
            fr->fb, precision, auto_block_frames(s->s->device(), fr->fb, lda, rsz), lda,
            [&](int64_t first, int64_t) -> void* { return base + (size_t)first * lda * rsz; },
            [](int64_t, int64_t, const void*) { return true; }, &s->last);
    });
}

int cg_assemble_stream(cg_session* s, const cg_frames* fr, int precision, int block_frames, cg_rows_sink sink,
                       void* user) {
    return guarded([&] {
        need(s && fr && sink, "session/frames/sink");
        need(precision == CG_FP64 || precision == CG_FP32, "precision");
        need(block_frames >= 0, "block_frames");
        const size_t rsz = precision == CG_FP64 ? 8 : 4;
        const int64_t lda = s->s->model().tot_all;
        const int bf = block_frames > 0 ? block_frames : auto_block_frames(s->s->device(), fr->fb, lda, rsz);
        int64_t maxrows = 1;
        for (int f0 = 0; f0 < fr->fb.nframes; f0 += bf) {
            const int f1 = std::min(fr->fb.nframes, f0 + bf);
            maxrows = std::max<int64_t>(maxrows, fr->fb.row_ofs[f1] - fr->fb.row_ofs[f0]);
        }
        const size_t bytes = (size_t)maxrows * lda * rsz;
        void* H[2] = {s->s->pinned(0, bytes), s->s->pinned(1, bytes)};
        int next = 0, rc = 0;
        s->s->assemble_to_host(
            fr->fb, precision, bf, lda, [&](int64_t, int64_t) -> void* { return H[next++ % 2]; },
            [&](int64_t first, int64_t nrows, const void* host) {
                rc = sink(user, first, nrows, host, lda);
                return rc == 0;
            },
            &s->last);
        if (rc != 0) throw cg::Error(1, "the row sink stopped the assembly (returned " + std::to_string(rc) + ")");
    });
}

int cg_session_last_counts(const cg_session* s, int64_t* pairs, int64_t* triplets, int64_t* quads, int64_t* evals3,
                           int64_t* evals4) {
    return guarded([&] {
        need(s, "session");
        if (pairs) *pairs = s->last.pairs2;
        if (triplets) *triplets = s->last.triplets;
        if (quads) *quads = s->last.quads;
        if (evals3) *evals3 = s->last.power_evals3;
        if (evals4) *evals4 = s->last.power_evals4;
    });
}

int cg_gram_weighted(cg_session* s, int a_precision, const void* A, int64_t lda, int64_t nrows, int ncols,
                     const double* b, const double* w, int mode, double* G, double* h) {
    return guarded([&] {
        need(s && A && b && w && G && h && ncols > 0 && lda >= ncols && nrows >= 0, "gram arguments");
        need(a_precision == CG_FP64 || a_precision == CG_FP32, "precision");
        need(mode == CG_GRAM_FP64 || mode == CG_GRAM_BF16X3, "gram mode");
        s->s->gram(a_precision, A, lda, nrows, ncols, b, mode, G, h, w);
    });
}

int cg_gram(cg_session* s, int a_precision, const void* A, int64_t lda, int64_t nrows, int ncols, const double* b,
            int mode, double* G, double* h) {
    return guarded([&] {
        need(s && A && b && G && h && ncols > 0 && lda >= ncols && nrows >= 0, "gram arguments");
        need(a_precision == CG_FP64 || a_precision == CG_FP32, "precision");
        need(mode == CG_GRAM_FP64 || mode == CG_GRAM_BF16X3, "gram mode");
        s->s->gram(a_precision, A, lda, nrows, ncols, b, mode, G, h);
    });
}

int cg_gram_finish(cg_session* s, double* G, int ncols) {
    return guarded([&] {
        need(s && G && ncols > 0, "gram_finish arguments");
        s->s->gram_finish(G, ncols);
    });
}

int cg_solve(cg_session* s, const double* G, const double* h, int ncols, double ridge, const double* A, int64_t lda,
             int64_t nrows, const double* b, int iters, double* x, double* info) {
    return guarded([&] {
        need(s && G && h && x && ncols > 0 && iters >= 0, "solve arguments");
        need(iters == 0 || (A && b && lda >= ncols), "refinement needs A and b");
        s->s->solve(G, h, ncols, ridge, A, lda, nrows, b, iters, x, info);
    });
}

int cg_solve_streamed(cg_session* s, const double* G, const double* h, int ncols, double ridge, int nblocks,
                      cg_dframes* const* blocks, const double* const* labels, const double* const* weights,
                      const double* extra_A, int64_t extra_rows, const double* extra_b, const double* extra_w,
                      int max_iters, double tol, double* x, double* info) {
    return guarded([&] {
        need(s && G && h && x && ncols > 0 && nblocks >= 0 && max_iters >= 0 && tol >= 0.0, "solve arguments");
        need(nblocks == 0 || (blocks && labels), "blocks/labels");
        need(extra_rows >= 0 && (extra_rows == 0 || (extra_A && extra_b)), "extra rows");
        std::vector<const cg::DeviceFrames*> bl;
        std::vector<const double*> lb, wt;
        for (int k = 0; k < nblocks; ++k) {
            need(blocks[k] && labels[k], "block/labels entry");
            bl.push_back(blocks[k]->d.get());
            lb.push_back(labels[k]);
            if (weights) {
                need(weights[k] != nullptr, "weights entry");
                wt.push_back(weights[k]);
            }
        }
        s->s->solve_streamed(G, h, ncols, ridge, bl, lb, wt, extra_A, extra_rows, extra_b, extra_w, max_iters, tol, x,
                             info);
    });
}

static std::vector<const cg::DeviceFrames*> block_list(int nblocks, cg_dframes* const* blocks) {
    need(nblocks == 0 || blocks, "blocks");
    std::vector<const cg::DeviceFrames*> bl;
    for (int k = 0; k < nblocks; ++k) {
        need(blocks[k] != nullptr, "block entry");
        bl.push_back(blocks[k]->d.get());
    }
    return bl;
}

int cg_cholesky(cg_session* s, const double* G, int ncols, double ridge, double* L, double* ridge_used) {
    return guarded([&] {
        need(s && G && L && ncols > 0, "cholesky arguments");
        const double r = s->s->factor(G, ncols, ridge, L);
        if (ridge_used) *ridge_used = r;
    });
}

int cg_cholesky_solve(cg_session* s, const double* L, int ncols, const double* h, double* x) {
    return guarded([&] {
        need(s && L && h && x && ncols > 0, "cholesky_solve arguments");
        s->s->factor_solve(L, ncols, h, x);
    });
}

int cg_refine_streamed(cg_session* s, const double* L, int ncols, double ridge, int nblocks,
                       cg_dframes* const* blocks, const double* const* labels, const double* const* weights,
                       const double* extra_A, int64_t extra_rows, const double* extra_b, const double* extra_w,
                       int max_iters, double tol, double* x, double* info) {
    return guarded([&] {
        need(s && L && x && ncols > 0 && nblocks >= 0 && max_iters >= 0 && tol >= 0.0, "refine arguments");
        need(nblocks == 0 || labels, "labels");
        need(extra_rows >= 0 && (extra_rows == 0 || (extra_A && extra_b)), "extra rows");
        std::vector<const cg::DeviceFrames*> bl = block_list(nblocks, blocks);
        std::vector<const double*> lb, wt;
        for (int k = 0; k < nblocks; ++k) {
            need(labels[k] != nullptr, "labels entry");
            lb.push_back(labels[k]);
            if (weights) {
                need(weights[k] != nullptr, "weights entry");
                wt.push_back(weights[k]);
            }
        }
        s->s->refine_streamed(L, ncols, ridge, bl, lb, wt, extra_A, extra_rows, extra_b, extra_w, max_iters, tol, x,
                              info);
    });
}

int cg_predict_streamed(cg_session* s, int nblocks, cg_dframes* const* blocks, const double* x, double* y) {
    return guarded([&] {
        need(s && x && y && nblocks >= 0, "predict arguments");
        s->s->predict_streamed(block_list(nblocks, blocks), x, y);
    });
}

int cg_fp64_fma_rate(cg_session* s, double* tflops) {
    return guarded([&] {
        need(s && tflops, "session/tflops");
        *tflops = s->s->fp64_fma_tflops();
    });
}

int cg_lars(cg_session* s, const double* G, const double* h, int ncols, int64_t nsamples, double alpha, int max_iter,
            double* x, double* info) {
    return guarded([&] {
        need(s && G && h && x && ncols > 0 && nsamples > 0 && alpha >= 0.0 && max_iter > 0, "lars arguments");
        s->s->lars(G, h, ncols, nsamples, alpha, max_iter, x, info);
    });
}

int cg_dlars(cg_session* s, const double* G, const double* h, int ncols, int64_t nsamples, double btb, double lambda,
             int lasso, const double* colsum, double bsum, int max_iter, double* x, double* info) {
    return guarded([&] {
        need(s && G && h && x && ncols > 0 && nsamples > 0 && lambda >= 0.0 && max_iter > 0, "dlars arguments");
        if (colsum)
            s->s->dlars_normalized(G, h, colsum, bsum, ncols, nsamples, btb, lambda, lasso, max_iter, x, info);
        else
            s->s->lars(G, h, ncols, nsamples, lambda, max_iter, x, info, lasso ? 2 : 1, btb);
    });
}

int cg_dlars_ex(cg_session* s, const double* G, const double* h, int ncols, int64_t nsamples, double btb,
                double lambda, int lasso, const double* colsum, double bsum, int max_iter, double max_norm,
                const char* restart_in, const char* restart_out, double* x, double* info) {
    return guarded([&] {
        need(s && G && h && x && ncols > 0 && nsamples > 0 && lambda >= 0.0 && max_iter > 0, "dlars arguments");
        const double mn = max_norm > 0.0 ? max_norm : 1.0e50;
        if (colsum)
            s->s->dlars_normalized(G, h, colsum, bsum, ncols, nsamples, btb, lambda, lasso, max_iter, x, info, mn,
                                   restart_in, restart_out);
        else
            s->s->lars(G, h, ncols, nsamples, lambda, max_iter, x, info, lasso ? 2 : 1, btb, mn, restart_in,
                       restart_out);
    });
}

int cg_session_last_launches(const cg_session* s, int64_t* launches) {
    return guarded([&] {
        need(s && launches, "session/launches");
        *launches = s->last.launches;
    });
}

int cg_session_profile(cg_session* s, int enable) {
    return guarded([&] {
        need(s, "session");
        s->s->reset_stage_totals();
        s->s->set_profiling(enable != 0);
    });
}

int cg_session_stage_times(cg_session* s, double* ms, int64_t* calls) {
    return guarded([&] {
        need(s, "session");
        static_assert(CG_NSTAGES == cg::ST_COUNT, "stage count");
        s->s->stage_totals(ms, calls);
    });
}

const char* cg_stage_name(int stage) { return cg::stage_name(stage); }

// ------------------------------------------------------------------ MD force
int cg_md_setup(cg_session* s, const double* x, int nx, int precision, int flags, double penalty_dist,
                double penalty_scale) {
    return guarded([&] {
        need(s && x, "session/x");
        need(precision == CG_FP64 || precision == CG_FP32, "precision");
        need((flags & ~CG_MD_ENERGY_OFFSETS) == 0, "flags");
        s->s->md_setup(x, nx, precision, (flags & CG_MD_ENERGY_OFFSETS) != 0, penalty_dist, penalty_scale);
    });
}

int cg_md_force_device(cg_session* s, const cg_dframes* d, double* forces, double* scalars) {
    return guarded([&] {
        need(s && d && forces && scalars, "session/frames/forces/scalars");
        s->s->md_force(*d->d, forces, scalars, &s->md_last);
    });
}

int cg_md_force(cg_session* s, const cg_frames* fr, double* forces, double* scalars) {
    return guarded([&] {
        need(s && fr && forces && scalars, "session/frames/forces/scalars");
        cudaStream_t st = s->s->stream();
        std::unique_ptr<cg::DeviceFrames> d = s->s->upload(fr->fb);
        const size_t nf = (size_t)fr->fb.natoms_total * 3, ns = (size_t)fr->fb.nframes * cgd::MD_NSCALAR;
        double* dF = nullptr;
        cg::cuda_check(cudaMallocAsync((void**)&dF, std::max<size_t>(1, nf + ns) * sizeof(double), st),
                       "cudaMallocAsync(forces)");
        try {
            s->s->md_force(*d, dF, dF + nf, &s->md_last);
            cg::cuda_check(cudaMemcpyAsync(forces, dF, nf * sizeof(double), cudaMemcpyDeviceToHost, st),
                           "cudaMemcpyAsync(forces)");
            cg::cuda_check(cudaMemcpyAsync(scalars, dF + nf, ns * sizeof(double), cudaMemcpyDeviceToHost, st),
                           "cudaMemcpyAsync(scalars)");
            cg::cuda_check(cudaFreeAsync(dF, st), "cudaFreeAsync(forces)");
            cg::cuda_check(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        } catch (...) {
            cudaFreeAsync(dF, st);
            cudaStreamSynchronize(st);
            throw;
        }
    });
}

int cg_md_nve(cg_session* s, cg_dframes* d, const double* mass, double dt_fs, int nsteps, double* velocities,
              double* forces, double* scalars_steps, double* ke_steps) {
    return guarded([&] {
        need(s && d && mass && velocities && forces, "session/frames/mass/velocities/forces");
        need(dt_fs > 0.0 && nsteps >= 0, "dt/nsteps");
        const double Tfs = 48.888;   // internal time unit in fs (src/functions.h:44)
        s->s->md_nve(*d->d, mass, dt_fs / Tfs, nsteps, velocities, forces, scalars_steps, ke_steps);
    });
}

int cg_frames_subtract_coulomb(cg_session* s, cg_frames* fr) {
    return guarded([&] {
        need(s && fr, "session/frames");
        s->s->subtract_coulomb(fr->fb);
    });
}

int cg_md_nvt(cg_session* s, cg_dframes* d, const double* mass, double dt_fs, int nsteps, int style,
              double temperature, double tau_fs, double* velocities, double* forces, double* scalars_steps,
              double* ke_steps, double* conserved_steps) {
    return guarded([&] {
        need(s && d && mass && velocities && forces, "session/frames/mass/velocities/forces");
        need(dt_fs > 0.0 && nsteps >= 0, "dt/nsteps");
        need(style == CG_NVT_MTK || style == CG_NVT_BEREND || style == CG_NVT_SCALE, "thermostat style");
        const double Tfs = 48.888;   // internal time unit in fs (src/functions.h:44)
        cg::MdThermostat th;
        th.style = style == CG_NVT_MTK ? 1 : (style == CG_NVT_BEREND ? 2 : 6);
        th.temperature = temperature;
        th.tau_fs = tau_fs;
        s->s->md_run(*d->d, mass, dt_fs / Tfs, nsteps, th, velocities, forces, scalars_steps, ke_steps,
                     conserved_steps);
    });
}

int cg_md_npt(cg_session* s, cg_dframes* d, const double* mass, double dt_fs, int nsteps, int style,
              double temperature, double tau_fs, double pressure_gpa, double tau_baro_fs, double* velocities,
              double* forces, double* scalars_steps, double* ke_steps, double* conserved_steps,
              double* volume_steps) {
    return guarded([&] {
        need(s && d && mass && velocities && forces, "session/frames/mass/velocities/forces");
        need(dt_fs > 0.0 && nsteps >= 0, "dt/nsteps");
        need(style == CG_NPT_BEREND || style == CG_NPT_BEREND_ANISO || style == CG_NPT_MTK, "barostat style");
        cg::MdThermostat th;
        th.style = style;   // 3, 4, 5 as MdThermostat numbers them
        th.temperature = temperature;
        th.tau_fs = tau_fs;
        th.pressure_gpa = pressure_gpa;
        th.tau_baro_fs = tau_baro_fs;
        s->s->md_run(*d->d, mass, dt_fs / 48.888, nsteps, th, velocities, forces, scalars_steps, ke_steps,
                     conserved_steps, volume_steps);
    });
}

int cg_md_numerical(cg_session* s, const cg_frames* fr, int what, double* out) {
    return guarded([&] {
        need(s && fr && out && (what == 0 || what == 1), "session/frames/out/what");
        s->s->md_numerical(fr->fb, what == 1, out);
    });
}

int cg_md_write_traj(const cg_model* h, int format, const char* path, int frame_index, int step, double dt_fs,
                     double temperature, int wrap, int natoms, const int* types, const double* xyz,
                     const double* velocities, const double* cell) {
    return guarded([&] {
        need(h && path && types && xyz && cell && natoms >= 0 && frame_index >= 0, "model/path/arrays");
        need(format == CG_TRAJ_GEN || format == CG_TRAJ_XYZ || format == CG_TRAJ_LAMMPSTRJ, "trajectory format");
        cg::MdConfig c{natoms, types, xyz, velocities, cell};
        cg::write_traj_frame(h->m, (cg::TrajFormat)format, path, frame_index, step, dt_fs, temperature, wrap != 0, c);
    });
}

int cg_md_write_xyzv(const cg_model* h, const char* path, int natoms, const int* types, const double* xyz,
                     const double* velocities, const double* cell, int wrap) {
    return guarded([&] {
        need(h && path && types && xyz && velocities && cell && natoms >= 0, "model/path/arrays");
        cg::MdConfig c{natoms, types, xyz, velocities, cell};
        cg::write_xyzv(h->m, path, c, wrap != 0, nullptr, 0, 0.0, nullptr, nullptr);
    });
}

int cg_md_write_restart(cg_session* s, int frame, const char* path, int natoms, const int* types, const double* xyz,
                        const double* velocities, const double* accel, const double* cell, int step,
                        double rcut_padding, const double* avg7, int wrap) {
    return guarded([&] {
        need(s && path && types && xyz && velocities && accel && cell && natoms >= 0, "session/path/arrays");
        const std::vector<double> c29 = s->s->md_restart_fields(frame);
        cg::MdConfig c{natoms, types, xyz, velocities, cell};
        cg::write_xyzv(s->s->model(), path, c, wrap != 0, accel, step + 1, rcut_padding, c29.data(), avg7);
    });
}

int cg_md_read_restart(const cg_model* h, const char* path, int natoms, int* types, double* xyz,
                       double* velocities, double* accel, double* cell, int* step, double* rcut_padding,
                       double* constraint29, double* avg7) {
    return guarded([&] {
        need(h && path, "model/path");
        cg::MdRestart r = cg::read_restart(h->m, path);
        need((int)r.types.size() == natoms, "natoms (does not match the restart file)");
        if (types) std::copy(r.types.begin(), r.types.end(), types);
        if (xyz) std::copy(r.xyz.begin(), r.xyz.end(), xyz);
        if (velocities) std::copy(r.v.begin(), r.v.end(), velocities);
        if (accel) std::copy(r.acc.begin(), r.acc.end(), accel);
        if (cell) std::copy(r.cell, r.cell + 9, cell);
        if (step) *step = r.step;
        if (rcut_padding) *rcut_padding = r.rcut_padding;
        if (constraint29) std::copy(r.constraint, r.constraint + cg::RESTART_CONSTRAINT_FIELDS, constraint29);
        if (avg7) std::copy(r.avg, r.avg + cg::RESTART_AVG_FIELDS, avg7);
    });
}

int cg_md_velocities(int natoms, const double* mass, int generate, int seed, double temperature, double* v) {
    return guarded([&] {
        need(natoms >= 0 && (natoms == 0 || (mass && v)), "natoms/mass/v");
        cg::md_velocities(natoms, mass, generate != 0, seed, temperature, v);
    });
}

int cg_md_resume(cg_session* s, int nframes, const double* constraint29) {
    return guarded([&] {
        need(s && nframes >= 0, "session/nframes");
        s->s->md_resume(nframes, constraint29);
    });
}

int cg_md_serve(cg_session* s, int nreq, const cg_md_request* req, const double* mass, double dt_fs,
                double hbm_budget_bytes, int64_t max_batch_atoms, int max_batch_frames, cg_md_result* results,
                double* step_ms, int64_t* batch_steps) {
    return guarded([&] {
        need(s && (req || nreq == 0) && mass && results && nreq >= 0, "session/requests/mass/results");
        need(dt_fs > 0.0 && max_batch_atoms > 0 && max_batch_frames > 0 && hbm_budget_bytes > 0.0, "limits");
        std::vector<cg::MdRequest> rq(nreq);
        for (int r = 0; r < nreq; ++r) {
            rq[r].natoms = req[r].natoms; rq[r].nsteps = req[r].nsteps; rq[r].arrival = req[r].arrival;
            rq[r].types = req[r].types; rq[r].xyz = req[r].xyz; rq[r].cell = req[r].cell; rq[r].v = req[r].v;
            rq[r].xyz_out = req[r].xyz_out;
        }
        cg::MdServeOptions opt;
        opt.dt = dt_fs / 48.888;   // internal time unit in fs (src/functions.h:44)
        opt.hbm_budget = hbm_budget_bytes;
        opt.max_batch_atoms = max_batch_atoms;
        opt.max_batch_frames = max_batch_frames;
        std::vector<cg::MdResult> out(nreq);
        const int64_t nb = s->s->md_serve(rq, mass, opt, out.data(), step_ms);
        for (int r = 0; r < nreq; ++r) {
            results[r].admitted = out[r].admitted; results[r].finished = out[r].finished;
            results[r].step_ms_sum = out[r].step_ms_sum; results[r].step_ms_max = out[r].step_ms_max;
            results[r].reserved_bytes = out[r].reserved_bytes;
        }
        if (batch_steps) *batch_steps = nb;
    });
}

int cg_md_server_start(cg_session* s, const double* mass, double dt_fs, double hbm_budget_bytes,
                       int64_t max_batch_atoms, int max_batch_frames, cg_md_server** out) {
    return guarded([&] {
        need(s && mass && out, "session/mass/out");
        need(dt_fs > 0.0 && max_batch_atoms > 0 && max_batch_frames > 0 && hbm_budget_bytes > 0.0, "limits");
        cg::MdServeOptions opt;
        opt.dt = dt_fs / 48.888;   // internal time unit in fs (src/functions.h:44)
        opt.hbm_budget = hbm_budget_bytes;
        opt.max_batch_atoms = max_batch_atoms;
        opt.max_batch_frames = max_batch_frames;
        std::unique_ptr<cg_md_server> h(new cg_md_server());
        h->srv.reset(new cg::MdServer(*s->s, mass, opt));
        *out = h.release();
    });
}

int cg_md_server_submit(cg_md_server* srv, const cg_md_request* req, int64_t* ticket) {
    return guarded([&] {
        need(srv && req && ticket, "server/request/ticket");
        cg::MdRequest q;
        q.natoms = req->natoms; q.nsteps = req->nsteps; q.arrival = 0.0;
        q.types = req->types; q.xyz = req->xyz; q.cell = req->cell; q.v = req->v; q.xyz_out = nullptr;
        *ticket = srv->srv->submit(q);
    });
}

int cg_md_server_poll(cg_md_server* srv, int64_t ticket, int wait, cg_md_result* result, double* xyz_out) {
    int rc = 0;
    const int g = guarded([&] {
        need(srv, "server");
        cg::MdResult r;
        rc = srv->srv->poll(ticket, wait != 0, &r, xyz_out);
        if (rc == 0 && result) {
            result->admitted = r.admitted; result->finished = r.finished;
            result->step_ms_sum = r.step_ms_sum; result->step_ms_max = r.step_ms_max;
            result->reserved_bytes = r.reserved_bytes;
        }
    });
    return g ? g : rc;
}

int cg_md_server_stop(cg_md_server* srv, int64_t* batch_steps) {
    return guarded([&] {
        need(srv, "server");
        std::unique_ptr<cg_md_server> h(srv);   // freed on every path
        const int64_t nb = h->srv->stop();
        if (batch_steps) *batch_steps = nb;
    });
}

int cg_md_serve_memory(cg_session* s, int64_t max_batch_atoms, int max_batch_frames, double* arena_bytes,
                       double* bytes_per_atom) {
    return guarded([&] {
        need(s && max_batch_atoms > 0 && max_batch_frames > 0, "session/limits");
        s->s->md_serve_memory(max_batch_atoms, max_batch_frames, arena_bytes, bytes_per_atom);
    });
}

int cg_dframes_positions(const cg_dframes* d, double** xyz, int64_t* natoms) {
    return guarded([&] {
        need(d && xyz && natoms, "frames/xyz/natoms");
        *xyz = d->d->xyz;
        *natoms = d->d->natoms_total;
    });
}

int cg_dframes_read_positions(const cg_dframes* d, double* xyz_host) {
    return guarded([&] {
        need(d && xyz_host, "frames/xyz");
        cg::cuda_check(cudaMemcpy(xyz_host, d->d->xyz, 3 * d->d->natoms_total * sizeof(double), cudaMemcpyDeviceToHost),
                       "cudaMemcpy(positions)");
    });
}

int cg_md_last_counts(const cg_session* s, int64_t* pairs, int64_t* triplets, int64_t* quads, int64_t* launches) {
    return guarded([&] {
        need(s, "session");
        if (pairs) *pairs = s->md_last.pairs2;
        if (triplets) *triplets = s->md_last.triplets;
        if (quads) *quads = s->md_last.quads;
        if (launches) *launches = s->md_last.launches;
    });
}

// ------------------------------------------------------------------ batched fit
int cg_batch_fit_create(cg_session* s, int nblocks, cg_dframes* const* blocks, const double* const* labels,
                        int a_precision, void* A, int64_t lda, double* G, double* h, cg_batch_fit** out) {
    return guarded([&] {
        need(s && blocks && labels && A && G && h && out && nblocks > 0, "batch fit arguments");
        need(a_precision == CG_FP64 || a_precision == CG_FP32, "precision");
        std::vector<const cg::DeviceFrames*> bl(nblocks);
        std::vector<const double*> lb(nblocks);
        std::vector<cg::RunPlan> plans(nblocks);
        for (int k = 0; k < nblocks; ++k) {
            need(blocks[k] && labels[k], "block");
            bl[k] = blocks[k]->d.get();
            lb[k] = labels[k];
            plans[k] = s->s->plan(*bl[k], a_precision, A, lda);   // sizing pass
        }
        std::unique_ptr<cg_batch_fit> o(new cg_batch_fit());
        o->b = s->s->batch_fit_graph(bl, plans, lb, a_precision, A, lda, G, h);
        *out = o.release();
    });
}

int cg_batch_fit_launch(cg_session* s, cg_batch_fit* b) {
    return guarded([&] {
        need(s && b, "session/batch");
        s->s->batch_fit_launch(*b->b);
    });
}

int cg_batch_fit_nodes(const cg_batch_fit* b, int64_t* nodes) {
    return guarded([&] {
        need(b && nodes, "batch/nodes");
        *nodes = b->b->nodes;
    });
}

void cg_batch_fit_free(cg_batch_fit* b) { delete b; }

int cg_session_tune(cg_session* s, const char* key, int value) {
    return guarded([&] {
        need(s && key, "session/key");
        const std::string k(key);
        if (k == "gram_ctas_per_sm") s->s->set_gram_ctas_per_sm(value);
        else if (k == "md_skin_milli") s->s->set_md_skin(value * 1e-3);
        else if (k == "gram_rows_per_launch") s->s->set_gram_rows_per_launch(value);
        else if (k == "force4_threads") s->s->set_force4_threads(value);
        else if (k == "force_range") s->s->set_force_range(value);
        else if (k == "host_staging") s->s->set_host_staging(value);
        else if (k == "cholesky_tensor_updates") s->s->set_cholesky_tensor_updates(value != 0);
        else if (k == "refine_cache_mb") s->s->set_refine_cache_bytes(value < 0 ? -1 : (int64_t)value << 20);
        else throw cg::Error(1, "unknown tuning key: " + k);
    });
}

}  // extern "C"
