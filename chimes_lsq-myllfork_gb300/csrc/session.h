// Host orchestration of the design-matrix path on one GPU: device copies of the
// model tables, device-resident frame batches, and the launch sequence
//   ghosts -> neighbour lists -> clusters -> owner / type buckets -> A rows.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <functional>
#include <initializer_list>
#include <memory>
#include <string>
#include <vector>

#include "dev.cuh"
#include "md.h"
#include "model.h"

namespace cg {

struct Scratch;
void cuda_check(cudaError_t e, const char* what);

// Model tables uploaded to the device (immutable after creation).
struct DeviceModel {
    cgd::ModelDev dev{};
    std::vector<void*> allocs;
    int max_allowed3 = 0, max_allowed4 = 0;
    explicit DeviceModel(const Model& m, int vir_pchunk);
    ~DeviceModel();
    DeviceModel(const DeviceModel&) = delete;
    DeviceModel& operator=(const DeviceModel&) = delete;
};

// Host-side flattened frames (one A-matrix row block per frame).
struct FrameBatch {
    int nframes = 0, first_index = 0;
    std::vector<int> natoms, stress_rows, energy_rows;
    std::vector<int64_t> atom_ofs, ghost_ofs, row_ofs;
    std::vector<cgd::BoxDev> box;
    std::vector<int> type;
    std::vector<double> xyz;
    std::vector<double> b;        // labels in A row order (src/A_Matrix.C:294-553)
    std::vector<char> small_self; // each frame's own small-cell test (no carry-over)
    std::vector<int> file;        // trajectory file of each frame (b-labeled.txt flags)
    std::vector<int> rank;        // chimes_lsq rank whose output files hold the frame
    int nprocs = 1;               // ranks of that emulated run
    int64_t nrows = 0, natoms_total = 0, nghosts = 0;
};

// Frames carry their trajectory index (NSTRESS / NENER) when they have one, else
// first_index + position; nprocs is the rank count of an emulated chimes_lsq run.
FrameBatch make_batch(const Model& m, const std::vector<Frame>& frames, int first_index, int nprocs = 1);
// The small-cell convention is sticky along a trajectory (the fit reads frames in
// sequence); independent configurations (MD systems) each decide it alone.
void make_independent(FrameBatch& fb);
// Frames [first, first + count) of a batch (their carried-over small-cell state kept).
FrameBatch slice_batch(const FrameBatch& fb, int first, int count);
void set_small(cgd::BoxDev& bd, bool small);

// The same batch resident in device memory.
struct DeviceFrames {
    cgd::FramesDev dev{};
    int nframes = 0;
    int64_t nrows = 0, natoms_total = 0, nghosts = 0;
    std::vector<int64_t> atom_ofs_host, row_ofs_host;
    std::vector<int> natoms_host;
    std::vector<void*> allocs;
    double* xyz = nullptr;          // the positions dev.xyz points to (the MD updates them)
    std::vector<cgd::BoxDev> box_host;   // host copy of the boxes (binned neighbour search)
    ~DeviceFrames();
};

struct AssembleStats {
    int64_t pairs2 = 0, list3 = 0, list4 = 0, triplets = 0, quads = 0;
    int64_t power_evals3 = 0, power_evals4 = 0;   // sum over clusters of n_allowed
    int64_t launches = 0;                         // kernels launched by the last call
};

// Coefficient tables of the MD force (md.h), built from one fitted vector x.
struct MdTables {
    cgd::MdDev dev{};
    int precision = 0;                 // 0: FP64 contraction, 1: FP32 contraction
    std::vector<void*> allocs;
    ~MdTables() { for (void* p : allocs) cudaFree(p); }
};

struct MdCounts {
    int64_t pairs2 = 0, triplets = 0, quads = 0, launches = 0;
};

// MD neighbour / cluster lists enumerated with a skin and reused over steps until
// an atom has moved more than skin / 2 (the cluster set of each step is still
// exact: a per-step filter keeps the clusters inside their cut-offs).
struct MdLists {
    std::vector<void*> allocs;            // grow-only buffers, one per slot, kept across rebuilds
    std::vector<size_t> caps;
    cgd::NeighDev NB{};
    cgd::ClusterSet CS[2]{};
    int64_t ncl[2] = {0, 0};
    int* tstep[2] = {nullptr, nullptr};   // per-step type (-1: out of range)
    int64_t* cfo[2] = {nullptr, nullptr};
    cgd::MdBuckets B[2]{};
    double* xref = nullptr;               // positions at the build
    int* shift = nullptr;                 // wrap shifts at the build
    double* scaled = nullptr;             // the build's own ghost coordinates, so that a
    float* cart32 = nullptr;              // build can run beside a force evaluation
    unsigned long long* dmax = nullptr;
    int64_t natoms = 0;
    double skin = 0.0;
    bool valid = false;
    int64_t builds = 0;
    void release() { valid = false; }     // the buffers stay for the next build
    void* buffer(int slot, size_t bytes);
    ~MdLists();
};

// The lists of a running MD batch and a second set built ahead of need: once an
// atom has moved 3/8 of the skin (lists stay valid up to 1/2), the next lists are
// built on a side stream while the current step's forces run on the main stream,
// and the following step switches to them; a rebuild then costs no step time.
struct MdListSet {
    MdLists lists[2];
    int cur = 0;
    bool next_ready = false;
    int64_t early_builds = 0;
    MdLists& current() { return lists[cur]; }
    void release() { lists[0].release(); lists[1].release(); next_ready = false; }
};

// Thermostat of an MD run: style 0 NVE, 1 NVT-MTK (Nose-Hoover chain of one, MTK
// integration), 2 NVT-BEREND; temperature in K, time constant in fs.
// style: 0 NVE, 1 NVT-MTK, 2 NVT-BEREND, 3 NPT-BEREND, 4 NPT-BEREND-ANISO, 5 NPT-MTK,
// 6 NVT-SCALE (CONSTRAINT::INITIALIZE src/ClassDefs.C:527-585); pressure in GPa, time
// constants in fs (NVT-SCALE: tau_fs holds the steps between rescalings).
struct MdThermostat {
    int style = 0;
    double temperature = 0.0, tau_fs = 0.0;
    double pressure_gpa = 0.0, tau_baro_fs = 0.0;
};

// One MD request of the serving loop (host arrays owned by the caller).
struct MdRequest {
    int natoms = 0, nsteps = 0;
    double arrival = 0.0;             // seconds after the start of the run
    const int* types = nullptr;
    const double* xyz = nullptr;
    const double* cell = nullptr;     // ax ay az bx by bz cx cy cz
    const double* v = nullptr;        // A per internal time unit
    double* xyz_out = nullptr;        // final positions (may be null)
};
struct MdResult {
    double admitted = 0, finished = 0;    // seconds after the start of the run
    double step_ms_sum = 0, step_ms_max = 0;
    double reserved_bytes = 0;            // device memory reserved for it at admission
};
struct MdServeOptions {
    double dt = 0;                        // internal time units
    double hbm_budget = 150e9;            // bytes of device memory requests may hold
    int64_t max_batch_atoms = 1 << 16;
    int max_batch_frames = 1024;
};

// Where the serving loop (Session::serve_loop) takes its requests from: the fixed
// list of cg_md_serve, or the queue that cg_md_server_submit fills while the loop
// runs.  Requests have dense ids 0, 1, 2, ... in the order the source offers them.
struct ServeSource {
    virtual ~ServeSource() = default;
    // The next request to admit if it has arrived by `now` (seconds on the loop's
    // clock), else -1.  The same id is offered again until admitted() is called.
    virtual int next(double now) = 0;
    virtual void admitted() = 0;
    virtual const MdRequest& request(int id) = 0;
    // Called when no request is running: waits until next() may offer one; false
    // when no request will come any more.
    virtual bool wait(double now) = 0;
    // Request id has finished: its final positions are in its xyz_out.
    virtual void finished(int id, const MdResult& r) = 0;
};

// Sizes of one batch's work lists, recorded by a sizing pass so that later passes
// over the same batch need no host synchronisation (CUDA-graph capture).
struct RunPlan {
    int64_t tot[3] = {0, 0, 0};   // 2-body pairs, 3-body and 4-body candidate lists
    int64_t ncl[2] = {0, 0};      // triplets, quadruplets
    int hmax[2] = {0, 0};         // largest (frame, type) group of each
};

// A batched fit captured as one CUDA graph: every block's assembly and its
// tensor-core Gram accumulation, replayed by one launch.
struct BatchFit {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int* d_err = nullptr;
    int64_t nodes = 0;
    ~BatchFit();
};

// Pipeline stages timed with CUDA events when profiling is on.
enum Stage {
    ST_SETUP = 0, ST_NEIGH, ST_CLUSTERS, ST_BUCKET, ST_FORCE2, ST_VIRIAL2, ST_FORCE3, ST_VIRIAL3, ST_FORCE4,
    ST_VIRIAL4, ST_OTHER, ST_GRAM_ATB, ST_GRAM_SPLIT, ST_GRAM_TC, ST_GRAM_SYRK, ST_REFINE_PRODUCTS,
    ST_REFINE_PRECOND, ST_HOST_COPY, ST_COUNT
};
const char* stage_name(int s);

class Session {
   public:
    Session(const Model& m, int device);
    ~Session();
    const Model& model() const { return model_; }
    cudaStream_t stream() const { return stream_; }
    std::unique_ptr<DeviceFrames> upload(const FrameBatch& fb);
    // A (device pointer, row-major, lda >= tot_all) receives the batch's rows.
    void assemble(const DeviceFrames& df, int precision, void* A, int64_t lda, AssembleStats* stats);
    // A host batch assembled in blocks of block_frames frames into host memory: block
    // k is assembled on the session stream while block k-1 is copied to the host on
    // a copy stream.  dest(first_row, nrows) names the host destination of a block
    // (row-major, lda = ldh); done(first_row, nrows, host) is called once its copy has
    // landed (before the destination of block k+1 is reused) and may return false
    // to stop.  Returns the rows assembled.
    int64_t assemble_to_host(const FrameBatch& fb, int precision, int block_frames, int64_t ldh,
                             const std::function<void*(int64_t, int64_t)>& dest,
                             const std::function<bool(int64_t, int64_t, const void*)>& done, AssembleStats* stats);
    // Pinned host staging buffer i (0 or 1) of at least `bytes`, kept and grown across
    // calls (streamed assemblies), freed with the session.
    void* pinned(int i, size_t bytes);
    // host staging of streamed row blocks: 0 = 512 MiB-aligned memory advised for huge
    // pages and registered with CUDA, 1 = cudaMallocHost (the default)
    void set_host_staging(int kind);
    // Same pipeline with every per-call device buffer taken from a fixed static
    // device array (no cudaMalloc / cudaMallocAsync / cudaFree in the call).
    void assemble_noalloc(const DeviceFrames& df, int precision, void* A, int64_t lda, AssembleStats* stats);

    // Normal equations (gram.cu / solve.cu) on the session stream.
    void gram(int prec_in, const void* A, int64_t lda, int64_t nrows, int ncols, const double* b, int mode, double* G,
              double* h, const double* w = nullptr);
    void gram_finish(double* G, int ncols);
    // x = (G + ridge I)^-1 h, then `iters` preconditioned-CG steps on A^T A x = A^T b
    // (A may be null when iters == 0).  info: [rnorm, gnorm, ridge used].
    void solve(const double* G, const double* h, int ncols, double ridge, const double* A, int64_t lda, int64_t nrows,
               const double* b, int iters, double* x, double* info);
    // The mixed form's solve without a stored FP64 A: x = (G + r I)^-1 h (FP64
    // Cholesky), then preconditioned CG on the FP64 ridge system whose products
    // A^T (A p) and residual A^T (b - A x) are formed block by block from FP64 rows
    // assembled again for each pass (labels[k], weights[k]: block k's b and row
    // weights on the device; weights may be empty).  extra_A (device, row-major,
    // extra_rows x ncols, may be null) joins as one more block (charge-constraint
    // rows).  Stops after max_iters passes or when the relative update reaches tol.
    // info: [iterations, last relative update, initial and final residual norm, r].
    void solve_streamed(const double* G, const double* h, int ncols, double ridge,
                        const std::vector<const DeviceFrames*>& blocks, const std::vector<const double*>& labels,
                        const std::vector<const double*>& weights, const double* extra_A, int64_t extra_rows,
                        const double* extra_b, const double* extra_w, int max_iters, double tol, double* x,
                        double* info);
    // Its pieces: L = FP64 Cholesky factor of G + r I (returns r; L: ncols^2 device
    // doubles), x = (L L^T)^-1 h, and the CG passes from a given x (info: iterations,
    // last relative update, initial and final residual norm).
    double factor(const double* G, int ncols, double ridge, double* L);
    void factor_solve(const double* L, int ncols, const double* h, double* x);
    void refine_streamed(const double* L, int ncols, double ridge, const std::vector<const DeviceFrames*>& blocks,
                         const std::vector<const double*>& labels, const std::vector<const double*>& weights,
                         const double* extra_A, int64_t extra_rows, const double* extra_b, const double* extra_w,
                         int max_iters, double tol, double* x, double* info);
    // y = A x for every row of the blocks (in block order), from FP64 rows assembled
    // block by block (chimes_lsq.py's force.txt without a stored A).
    void predict_streamed(const std::vector<const DeviceFrames*>& blocks, const double* x, double* y);
    // Sizing pass of a batch (a full assembly into A) recording its list sizes.
    RunPlan plan(const DeviceFrames& df, int precision, void* A, int64_t lda);
    // Capture the assembly of every block into Abuf (lda) and the split-BF16 Gram
    // accumulation into G, h (labels: each block's b on the device) as one graph.
    std::unique_ptr<BatchFit> batch_fit_graph(const std::vector<const DeviceFrames*>& blocks,
                                              const std::vector<RunPlan>& plans,
                                              const std::vector<const double*>& labels, int precision, void* Abuf,
                                              int64_t lda, double* G, double* h);
    void batch_fit_launch(BatchFit& bf);
    void set_gram_ctas_per_sm(int v) { gram_ctas_per_sm_ = v > 0 ? v : 4; }
    // Rows of A per tensor-core Gram launch (0: the default of about 1 GiB of BF16
    // planes).  Each launch sums its rows in FP32 before adding into the FP64 G, so
    // the accumulation error grows with this length (diagonal entries linearly).
    void set_gram_rows_per_launch(int64_t v) { gram_rows_per_launch_ = v > 0 ? v : 0; }
    // Bytes of FP64 row blocks the streamed refinement may keep resident between
    // passes (-1: what the device has free beyond a margin; 0: none).
    void set_refine_cache_bytes(int64_t v) { refine_cache_bytes_ = v; }
    // Threads per CTA of the 4-body force kernel (512 or 1024).
    void set_force4_threads(int v) { force4_threads_ = v == 1024 ? 1024 : 512; }
    // many-body force rows: the range form (k_force_rg) never (0); in FP64, and in FP32
    // where a cluster type has more allowed powers than MB_THREADS (1, the default);
    // or always (2); else the per-power form k_force_mb
    void set_force_range(int v) { force_range_ = v < 0 ? 0 : (v > 2 ? 2 : v); }
    // Cholesky trailing updates by exact BF16 digit products on the tensor cores
    // (FP64-accurate) or by the FP64 SYRK.
    void set_cholesky_tensor_updates(bool v) { chol_tensor_ = v; }
    int gram_ctas_per_sm() const { return gram_ctas_per_sm_; }
    int device() const { return device_; }
    // Measured FP64 FMA rate of the session's GPU in TFLOP/s (dense64.cu).
    double fp64_fma_tflops();
    // LARS-lasso on the normal equations (lars.cu).
    void lars(const double* G, const double* h, int ncols, int64_t nsamples, double alpha, int max_iter, double* x,
              double* info, int mode = 0, double btb = 0.0, double max_norm = 1.0e50, const char* restart_in = nullptr,
              const char* restart_out = nullptr);
    // DLARS with column normalisation (colsum = A^T 1 on the device, bsum = sum b).
    void dlars_normalized(const double* G, const double* h, const double* colsum, double bsum, int ncols,
                          int64_t nsamples, double btb, double lambda, int lasso, int max_iter, double* x, double* info,
                          double max_norm = 1.0e50, const char* restart_in = nullptr,
                          const char* restart_out = nullptr);

    // MD force (md.h / md_host.cu).  md_setup stores the coefficients x (one per A
    // column): offsets adds the per-atom-type energy offsets of an energy fit.
    void md_setup(const double* x, int nx, int precision, bool offsets, double pen_dist, double pen_scale);
    bool md_ready() const { return (bool)md_; }
    // Forces Fo [natoms_total*3] and per-frame scalars So [nframes*MD_NSCALAR]
    // (device pointers) of the batch's current positions.
    void md_force(const DeviceFrames& df, double* Fo, double* So, MdCounts* counts);
    // Skin lists: build, force with the lists (no host synchronisation), and the
    // rebuild test (reads the largest displacement since the build).
    void md_lists_build(DeviceFrames& df, double skin, MdLists& L, cudaStream_t st);
    void md_force_lists(DeviceFrames& df, MdLists& L, double* Fo, double* So);
    double md_lists_disp2(const DeviceFrames& df, MdLists& L);   // largest squared displacement
    // One step's forces through a list set (rebuilds, look-ahead builds, switch).
    void md_force_step(DeviceFrames& df, MdListSet& LS, double* Fo, double* So);
    // Thermostat / barostat state of frame `frame` after the last md_run as CONSTRAINT's
    // 29 restart values (CONSTRAINT::WRITE order, src/ClassDefs.C:790-827); values a
    // device run does not track (the last Berendsen scale factors, KIN_ENER) hold what
    // a fresh CONSTRAINT holds.
    std::vector<double> md_restart_fields(int frame) const;
    // The next md_run starts every frame from these restart values (nframes x 29,
    // CONSTRAINT::READ): thermostat and barostat positions, velocities, forces and
    // inertias.
    void md_resume(int nframes, const double* constraint29);
    // Finite-difference pressure / stress of each frame (PRSCALC / STRSCALC NUMERICAL,
    // numerical_pressure and numerical_stress_all src/functions.C:402-628): the
    // strained replicas of every frame (cell and coordinates scaled by 1 +- 1e-4, or by
    // I +- 1e-4 e_i e_j) evaluated as one batch.  out: one PRESSURE_XYZ per frame
    // (stress false) or nine PRESSURE_TENSORS_XYZ_ALL entries per frame (row-major).
    void md_numerical(const FrameBatch& fb, bool stress, double* out);
    double md_skin() const { return md_skin_; }
    void set_md_skin(double s) { md_skin_ = s >= 0.0 ? s : 0.0; }
    // nsteps velocity-Verlet steps (NVE) of every frame of the batch; df's positions
    // and v [natoms_total*3] (device) are advanced in place.  mass_type: host,
    // natmtyp masses.  So_steps [(nsteps+1)*nframes*MD_NSCALAR] and ke_steps
    // [(nsteps+1)*nframes] (device, may be null) receive step 0..nsteps.
    // Fixed charges (FITCOUL false, ATMCHRG != 0): subtract each frame's Ewald
    // forces from its force labels (SubtractEwaldForces src/Ewald.C:827-845, called
    // by process_frame src/chimes_lsq.C:800-801), with the Ewald parameters of the
    // run's first frame (ZCalc_Ewald keeps them in statics).
    void subtract_coulomb(FrameBatch& fb);
    void md_nve(DeviceFrames& df, const double* mass_type, double dt, int nsteps, double* v, double* Fo,
                double* So_steps, double* ke_steps);
    // The same loop with a thermostat (CONSRNT NVT-MTK HOOVER tau / NVT-BEREND tau);
    // cons_steps ((nsteps+1) * nframes, device, may be null) receives the
    // thermostat's conserved-quantity term (NVT-MTK).
    void md_run(DeviceFrames& df, const double* mass_type, double dt, int nsteps, const MdThermostat& th, double* v,
                double* Fo, double* So_steps, double* ke_steps, double* cons_steps, double* vol_steps = nullptr);
    // Continuous-batching serving loop: requests are admitted on arrival while the
    // batch has room (atoms, frames, memory budget), every batched step advances all
    // admitted requests by one velocity-Verlet step, finished requests leave at once.
    // step_ms (may be null): per (request, step) wall time of the batched step, stride
    // = largest nsteps.  Returns the number of batched steps.
    int64_t md_serve(const std::vector<MdRequest>& req, const double* mass_type, const MdServeOptions& opt,
                     MdResult* res, double* step_ms);
    // The loop itself, over any request source (step_ms as above, or null).
    int64_t serve_loop(ServeSource& src, const double* mass_type, const MdServeOptions& opt, double* step_ms,
                       int stride);
    // Checks one serving request against the model and the loop's capacities (throws
    // Error 1 / 2) and returns its device box.
    cgd::BoxDev serve_check(const MdRequest& q, const MdServeOptions& opt, const std::string& who) const;
    // Device memory of the loop's two arenas, and what a running request of `atoms`
    // atoms reserves for its lists.
    double serve_fixed_bytes(const MdServeOptions& opt) const;
    double serve_need_bytes(int64_t atoms) const { return 2.0 * serve_list_per_atom_ * (double)atoms; }
    // Device memory of the serving loop: the fixed bytes of its two arenas for these
    // capacities, and the bytes a request reserves per atom (list estimate; measured
    // by the last serving run of this session, a prior before any).
    void md_serve_memory(int64_t max_batch_atoms, int max_batch_frames, double* arena, double* per_atom) const;

    // Stage timing (CUDA events on the session stream).
    void set_profiling(bool on) { profiling_ = on; }
    void stage_totals(double* ms, int64_t* calls);   // syncs pending events, accumulates, returns totals
    void reset_stage_totals();
    void mark(int stage, bool begin);
    // Host reads of a few device bytes (sizes, error words) ordered on stream st: a
    // one-thread kernel stores them into mapped pinned memory, then the host waits
    // for st.  A copy-engine read would queue behind a large block copy on the copy
    // stream and serialise the assembly with it.  At most 256 bytes per call.
    struct PeekItem { void* host; const void* dev; int bytes; };
    void peek(cudaStream_t st, std::initializer_list<PeekItem> items);

   private:
    void run(const DeviceFrames& df, int precision, void* A, int64_t lda, AssembleStats* stats, struct Scratch& S,
             const struct RunPlan* plan_in, struct RunPlan* plan_out);
    Model model_;
    bool profiling_ = false;
    struct Pending { int stage; cudaEvent_t a, b; };
    std::vector<Pending> pending_;
    std::vector<cudaEvent_t> event_pool_;
    double stage_ms_[ST_COUNT] = {0};
    int64_t stage_calls_[ST_COUNT] = {0};
    cudaEvent_t open_event_ = nullptr;
    int open_stage_ = -1;
    int device_;
    int sms_ = 1;   // streaming multiprocessors of the device
    cudaStream_t stream_ = nullptr;
    cudaStream_t side_stream_ = nullptr;   // look-ahead MD list builds
    cudaStream_t copy_stream_ = nullptr;   // device-to-host copies of streamed assemblies
    void* pinned_[2] = {nullptr, nullptr};
    size_t pinned_bytes_[2] = {0, 0};
    bool pinned_reg_[2] = {false, false};   // registered host memory (else cudaMallocHost)
    bool staging_huge_ = false;             // staging from huge-page registered memory
    unsigned char* mailbox_host_ = nullptr;   // mapped pinned bytes written by peek()
    unsigned char* mailbox_dev_ = nullptr;
    cudaEvent_t side_event_ = nullptr;
    cudaStream_t md_side_[2] = {nullptr, nullptr};   // many-body MD force parts beside the 2-body kernel
    cudaEvent_t md_fork_ = nullptr, md_join_[2] = {nullptr, nullptr};
    std::unique_ptr<DeviceModel> dm_;
    std::unique_ptr<MdTables> md_;
    int gram_ctas_per_sm_ = 4;
    int64_t gram_rows_per_launch_ = 0;
    int64_t refine_cache_bytes_ = -1;
    int force4_threads_ = 512;
    int force_range_ = 1;
    bool chol_tensor_ = true;
    int64_t gram_plane_rows(int64_t nrows, int ncols) const;
    double md_skin_ = 0.5;   // Angstrom; 0: enumerate every step
    std::atomic<double> serve_list_per_atom_{6144.0};   // list bytes per atom (measured by the serving loop)
    std::vector<double> md_state_;   // last md_run: nframes * MD_TH_STRIDE
    MdThermostat md_last_th_;
    std::vector<double> md_resume_;  // next md_run's starting restart values (nframes * 29)
};

}  // namespace cg
