/*
 * chimes_gb300 — C ABI of the GB300 design-matrix path of ChIMES-lsq.
 *
 * The reference has no FFI: its operator surface is the `chimes_lsq` CLI and the
 * in-process calls it makes.  Each entry point below replaces one step of that
 * surface (reference file:line cited beside it).  All entry points return 0 on
 * success and a non-zero status otherwise (1 bad argument, 2 bad input / unsupported
 * option, 3 CUDA failure, 4 out of memory); cg_last_error() returns the message of
 * the calling thread's last failure.  Handles are opaque; every buffer is owned by
 * the caller.  A session owns one CUDA stream and may be used by one thread at a time.
 */
#ifndef CHIMES_GB300_H
#define CHIMES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cg_model cg_model;
typedef struct cg_frames cg_frames;
typedef struct cg_session cg_session;
typedef struct cg_dframes cg_dframes;

/* Precision of the assembled A matrix. */
enum { CG_FP64 = 0, CG_FP32 = 1 };

/* Parse fm_setup.in and build the pair / cluster topology and coefficient map.
 * Replaces INPUT::PARSE_INFILE_LSQ (src/input.C:172-225), build_clusters
 * (src/chimes_lsq.C:533-560) and the column bookkeeping (src/chimes_lsq.C:198-248). */
int cg_model_load(const char* fm_setup_path, cg_model** out);
void cg_model_free(cg_model* m);

/* Column counts: 2-body, 3-body, 4-body, energy-offset and total A columns
 * (TOT_SNUM, NUM_3B_CHEBY, NUM_4B_CHEBY, TOT_ALL_PARAMS in src/chimes_lsq.C:198-248). */
int cg_model_columns(const cg_model* m, int* n2b, int* n3b, int* n4b, int* nener, int* ntotal);

/* FITCOUL (src/Ewald.C:477-750, src/A_Matrix.C:249-288): ncoul charge columns (one
 * q_i q_j product per pair type, after the short-range columns, before the energy
 * columns) and the number of CHARGE CONSTRAINTS rows (src/input.C:1148-1200). */
int cg_model_charge_columns(const cg_model* m, int* ncoul, int* nconstraints);

/* The charge-constraint rows that follow the last frame of a FITCOUL fit
 * (A_MAT::PRINT_CONSTRAINTS src/A_Matrix.C:569-625): nconstraints rows of A
 * (row-major, lda >= total columns) and their b values. */
int cg_model_constraint_rows(const cg_model* m, double* A, int64_t lda, double* b);

/* Rows a frame contributes after its 3 * natoms force rows, for frames below
 * NSTRESS / NENER: stress rows (0, 3 with FITSTRS true / FIRST: xx yy zz, 9 with ALL /
 * FIRSTALL: xx xy xz xy yy yz xz yz zz) and energy rows (0, or 3 identical rows with
 * FITENER) -- the row layout of A_MAT::PRINT_FRAME (src/A_Matrix.C:309-553). */
int cg_model_row_layout(const cg_model* m, int* stress_rows, int* energy_rows);

/* Number of frames (NFRAMES) and atom types (NATMTYP) of the model. */
int cg_model_sizes(const cg_model* m, int* nframes, int* natmtyp);

/* Text of params.header / ff_groups.map.  Writes at most cap bytes (NUL terminated
 * when room) and the full length to *needed.  Replaces print_param_header and
 * print_map_file (src/chimes_lsq.C:562-716). */
int cg_model_header_text(const cg_model* m, char* buf, size_t cap, size_t* needed);
int cg_model_map_text(const cg_model* m, char* buf, size_t cap, size_t* needed);

/* Text of params.txt, the fitted force-field file, for coefficients x[0..nx) (nx =
 * the model's column count): `preamble` (the solver's "!" comment block, may be
 * NULL), the params.header echo, the 2-body / cluster coefficient blocks, the
 * ff_groups.map text and the energy offsets, then ENDFILE.  Same buffer rules as
 * cg_model_header_text.  Replaces the output half of src/chimes_lsq.py:284-672. */
int cg_model_params_text(const cg_model* m, const double* x, int nx, const char* preamble, char* buf, size_t cap,
                         size_t* needed);

/* The coefficient vector (A-column order, nx = the model's column count) of a
 * params.txt text written for this model: the inverse of cg_model_params_text,
 * as chimes_md reads its PRMFILE (src/chimes_md.C:1700-2300). */
int cg_model_params_read(const cg_model* m, const char* params_txt, double* x, int nx);

/* Read nframes frames of an .xyzf trajectory (path NULL: the model's TRJFILE,
 * nframes <= 0: NFRAMES).  Replaces FRAME::READ_XYZF (src/ClassDefs.C:2411-2683). */
int cg_frames_read(const cg_model* m, const char* xyzf_path, int nframes, cg_frames** out);

/* The model's trajectory as `srun -n nprocs chimes_lsq` processes it: the frames of
 * each rank in rank order (contiguous blocks, divide_atoms src/functions.C:182-222,
 * or SKPFRMS round-robin with skipping, src/chimes_lsq.C:305-317), each frame keeping
 * its trajectory index for NSTRESS / NENER.  cg_write_lsq_files then writes the
 * files that run leaves (rank-ordered b.txt / b-labeled.txt / natoms.txt; with
 * SPLITFI, A.%04d.txt and dim.%04d.txt per rank).  nprocs = 1 is cg_frames_read of
 * the model's TRJFILE with SKPFRMS applied. */
int cg_frames_read_ranks(const cg_model* m, int nprocs, cg_frames** out);

/* Build frames from arrays (no text parsing).  Per frame f: natoms[f] atoms with
 * types (index into the TYPEIDX order) and xyz (A), forces (Hartree/Bohr, as in
 * .xyzf), cell[9*f..] = the 9 cell-vector components ax ay az bx by bz cx cy cz,
 * stress[6*f..] = xx yy zz xy xz yz (GPa, may be NULL), energy[f] (may be NULL).
 * first_index is the global index of the first frame (NSTRESS / NENER use it). */
int cg_frames_create(const cg_model* m, int nframes, const int* natoms, const int* types, const double* xyz,
                     const double* forces, const double* cell, const double* stress, const double* energy,
                     int first_index, cg_frames** out);
void cg_frames_free(cg_frames* fr);

/* Rows of the A matrix for these frames and the total atom count. */
int cg_frames_rows(const cg_frames* fr, int64_t* nrows, int64_t* natoms);

/* A.txt, b.txt, b-labeled.txt, natoms.txt and dim.txt of the frames in directory
 * dir, with A (host, row-major, lda >= columns) as assembled for them: the files of
 * `chimes_lsq fm_setup.in` (A_MAT::PRINT_FRAME / CLEANUP_FILES,
 * src/A_Matrix.C:210-720; %.16e, three spaces after force-row entries, one after
 * stress / energy entries).  A NULL writes every file but the A files.  SPLITFI
 * models write A.%04d.txt / dim.%04d.txt per rank of the batch's emulated run
 * (CLEANUP_FILES src/A_Matrix.C:626-720). */
int cg_write_lsq_files(const cg_model* m, const cg_frames* fr, const double* A, int64_t lda, const char* dir);
/* (FITCOUL models: A holds the frames' rows; the charge-constraint rows are appended
 * to A.txt and b.txt after them, as the reference writes them.) */

/* Number of frames in a batch. */
int cg_frames_count(const cg_frames* fr, int* nframes);

/* Frames [first, first + count) of a batch as a new batch (rows, labels and the
 * small-cell state of the trajectory kept): for assembling a fit in row blocks. */
int cg_frames_slice(const cg_frames* fr, int first, int count, cg_frames** out);

/* Treat the frames as independent configurations: each decides the small-cell
 * neighbour convention (PERM_SCALE, src/ClassDefs.C:44-67) from its own box,
 * instead of the fit's carry-over along a trajectory.  For MD batches; no
 * counterpart in the reference, whose chimes_md runs one system. */
int cg_frames_independent(cg_frames* fr);

/* Label vector b in A row order (src/A_Matrix.C:294-553), nrows doubles. */
int cg_frames_labels(const cg_frames* fr, double* b);

/* One GPU session (device ordinal) for a model; owns a CUDA stream. */
int cg_session_create(const cg_model* m, int device, cg_session** out);
void cg_session_free(cg_session* s);

/* The session's CUDA stream (cudaStream_t), for callers that order their own work after it. */
void* cg_session_stream(cg_session* s);

/* Assemble the full A matrix of the frames into HOST memory A (row-major,
 * nrows x lda, lda >= ntotal) in CG_FP64 (double) or CG_FP32 (float).  Host->device
 * copies of the coordinates and the device->host copies of A happen inside: the
 * frames are assembled in blocks, each block's copy overlapping the next block's
 * assembly (pinned host memory lets the copies run asynchronously).
 * Replaces the per-frame loop process_frame -> ZCalc_Deriv -> Deriv_2B/3B/4B
 * (src/chimes_lsq.C:292-328, 718-823; src/functions.C:755-804; src/Cheby.C:709-1729). */
int cg_assemble(cg_session* s, const cg_frames* fr, int precision, void* A, int64_t lda);

/* Streamed assembly into host memory without a host buffer for the whole A: the
 * frames are assembled in blocks of block_frames frames (0: about 1 GiB of A per
 * block), block k on the GPU while block k-1 is copied to pinned host memory, and
 * sink(user, first_row, nrows, A_block, lda) is called on the calling thread with each
 * block in row order (A_block: nrows x lda values of the requested precision, valid
 * until the sink returns; lda = the model's column count).  A non-zero return from
 * the sink stops the assembly (status 1).  cg_assemble uses the same pipeline with
 * the caller's buffer as the destination.  This is the shape of chimes_lsq's frame
 * loop that prints A.txt as it goes (src/chimes_lsq.C:292-328, A_MAT::PRINT_FRAME
 * src/A_Matrix.C:210-567), for A matrices larger than host memory. */
typedef int (*cg_rows_sink)(void* user, int64_t first_row, int64_t nrows, const void* A_block, int64_t lda);
int cg_assemble_stream(cg_session* s, const cg_frames* fr, int precision, int block_frames, cg_rows_sink sink,
                       void* user);

/* Device-resident variant: upload the frames once, then assemble into a DEVICE
 * buffer A.  cg_assemble_device is asynchronous on the session stream. */
int cg_frames_upload(cg_session* s, const cg_frames* fr, cg_dframes** out);
void cg_dframes_free(cg_dframes* d);
int cg_assemble_device(cg_session* s, const cg_dframes* d, int precision, void* A_device, int64_t lda);

/* Allocation-free assembly (this entry point has no counterpart in the reference).
 * For callers that cannot allocate device memory while they run -- an MD engine or
 * serving loop that reserves its memory at start-up and forbids allocation inside a
 * step, or a host application that manages the device heap through its own pool --
 * this variant of cg_assemble_device takes every per-call work buffer (neighbour
 * lists, cluster lists, owner buckets, counters) from one fixed device array of
 * CG_NOALLOC_SCRATCH_BYTES compiled into the library, and calls no cudaMalloc,
 * cudaMallocAsync or cudaFree.  The caller still provides the uploaded frames and the
 * output A (device, row-major, lda >= ntotal).  Inputs whose work lists do not fit
 * are rejected with status 4 and a message naming the capacity; the earlier stages of
 * such a call have already run, so the contents of A after a status-4 return are
 * unspecified (neither zeroed nor complete).  The array exists
 * once per GPU that loads the library and stays allocated until the process exits.
 * The first call on a device looks up the array's device address (make that first
 * call before any stream capture).  Every call on a device shares the array and
 * overwrites it, so calls that overlap on the GPU (other threads, other sessions'
 * streams) race; serialise them.  Stage profiling is not available here. */
#define CG_NOALLOC_SCRATCH_BYTES (32u << 20)
int cg_assemble_device_noalloc(cg_session* s, const cg_dframes* d, int precision, void* A_device, int64_t lda);

/* Normal equations of the fit (replaces the SVD of chimes_lsq.py, src/chimes_lsq.py:169-214).
 * cg_gram accumulates G += A^T A (row-major ncols x ncols FP64, upper triangle until
 * cg_gram_finish mirrors it) and h += A^T b for a device A block (row-major, lda,
 * a_precision CG_FP64 or CG_FP32).  mode CG_GRAM_FP64: FP64 SYRK on the CUDA cores (FP64 A);
 * CG_GRAM_BF16X3: A split into BF16 hi/lo planes, G from hi.hi + hi.lo + lo.hi on the
 * tensor cores with FP32 accumulation.  The caller zeroes G and h before the first
 * block.  All pointers are device pointers. */
enum { CG_GRAM_FP64 = 0, CG_GRAM_BF16X3 = 1 };
int cg_gram(cg_session* s, int a_precision, const void* A, int64_t lda, int64_t nrows, int ncols, const double* b,
            int mode, double* G, double* h);
int cg_gram_finish(cg_session* s, double* G, int ncols);

/* cg_gram with row weights w (device, nrows): G += (W A)^T (W A), h += (W A)^T (W b),
 * W = diag(w), as chimes_lsq.py --weights scales the rows of A and b
 * (src/chimes_lsq.py:140-149). */
int cg_gram_weighted(cg_session* s, int a_precision, const void* A, int64_t lda, int64_t nrows, int ncols,
                     const double* b, const double* w, int mode, double* G, double* h);

/* Ridge least squares (A^T A + ridge I) x = A^T b.  First x = (G + r I)^-1 h by FP64
 * Cholesky with r = ridge (r grows tenfold, at most 8 times, while G + r I is not
 * positive definite, as a mixed-precision G can be), then `iters` iterations of
 * conjugate gradients on the FP64 system (A^T A + ridge I) x = A^T b with products
 * through A, preconditioned by that factor -- so a tensor-core G converges to the
 * FP64 solution of the same system (A: FP64 device matrix; may be NULL if iters == 0).
 * info (host, 3 doubles): ||b - A x||, ||A^T (b - A x) - ridge x|| (0 when iters == 0),
 * and the r of the factorisation. */
int cg_solve(cg_session* s, const double* G, const double* h, int ncols, double ridge, const double* A, int64_t lda,
             int64_t nrows, const double* b, int iters, double* x, double* info);

/* The mixed form's ridge solve without a stored FP64 A (replaces the solve of
 * src/chimes_lsq.py:169-214 for a tensor-core Gram).  G, h: the normal equations of
 * the fit (device; typically the split-BF16 Gram of an FP32-assembled A).  First
 * x = (G + r I)^-1 h by FP64 Cholesky (r = ridge, grown as in cg_solve), then
 * preconditioned conjugate gradients on the FP64 system (A^T A + ridge I) x = A^T b:
 * every pass re-assembles each of the nblocks uploaded row blocks in FP64 into one
 * block-sized device buffer and folds it into A^T (A p) (or A^T (b - A x)), so no
 * FP64 A is ever stored whole.  labels[k] (device, block k's rows): b; weights
 * (NULL, or device row weights per block): rows enter as W A, W b
 * (src/chimes_lsq.py:140-149).  extra_A (device, row-major, extra_rows x ncols, may
 * be NULL with extra_rows 0), extra_b, extra_w (may be NULL): rows outside the
 * frames (FITCOUL charge constraints).  Stops after max_iters passes or once the
 * relative size of the last update |alpha| ||p|| / ||x|| falls to tol.  info (host, 5
 * doubles, may be NULL): passes made, last relative update, initial and final norm
 * of A^T (b - A x) - ridge x, and the r of the factorisation.  x: device, ncols. */
int cg_solve_streamed(cg_session* s, const double* G, const double* h, int ncols, double ridge, int nblocks,
                      cg_dframes* const* blocks, const double* const* labels, const double* const* weights,
                      const double* extra_A, int64_t extra_rows, const double* extra_b, const double* extra_w,
                      int max_iters, double tol, double* x, double* info);

/* The pieces of cg_solve_streamed, for callers that keep the factor: cg_cholesky
 * writes the FP64 Cholesky factor of G + r I into L (device, ncols * ncols doubles;
 * its column-major lower triangle; r = ridge grown as in cg_solve, returned in
 * *ridge_used, which may be NULL); cg_cholesky_solve: x = (L L^T)^-1 h;
 * cg_refine_streamed: the conjugate-gradient passes of cg_solve_streamed from the
 * caller's x (device, updated in place), preconditioned by L; info (4 doubles, may
 * be NULL): passes, last relative update, initial and final residual norm. */
int cg_cholesky(cg_session* s, const double* G, int ncols, double ridge, double* L, double* ridge_used);
int cg_cholesky_solve(cg_session* s, const double* L, int ncols, const double* h, double* x);
int cg_refine_streamed(cg_session* s, const double* L, int ncols, double ridge, int nblocks,
                       cg_dframes* const* blocks, const double* const* labels, const double* const* weights,
                       const double* extra_A, int64_t extra_rows, const double* extra_b, const double* extra_w,
                       int max_iters, double tol, double* x, double* info);

/* Predicted labels y = A x (device, one value per row of the blocks in order) from
 * FP64 rows assembled block by block: force.txt of chimes_lsq.py
 * (src/chimes_lsq.py:284-296) without a stored A. */
int cg_predict_streamed(cg_session* s, int nblocks, cg_dframes* const* blocks, const double* x, double* y);

/* FP64 fused multiply-add rate of the session's GPU in TFLOP/s (2 flops per FMA),
 * measured by a kernel of independent FMA chains on every SM (no counterpart in the
 * reference; the denominator of the FP64 roofline fractions).  Changes no device
 * setting. */
int cg_fp64_fma_rate(cg_session* s, double* tflops);

/* LARS with the lasso modification (the reference's `--algorithm lassolars`,
 * scikit-learn LassoLars with fit_intercept=False, src/chimes_lsq.py:248-263; the
 * active-set Cholesky updates of contrib/dlars/src/dlars.C:1101-1329) on the
 * normal equations: G (full symmetric after cg_gram_finish) and h = A^T b, device
 * FP64; nsamples = rows of A.  Minimises (1/2n)||b - A x||^2 + alpha ||x||_1 by
 * following the path to C / n = alpha exactly; x (device) receives the
 * coefficients.  info (host, 3 doubles, may be NULL): steps, active variables,
 * final C / n.  The active-set factor is updated by rank-1 additions and Givens
 * deletions in FP64. */
int cg_lars(cg_session* s, const double* G, const double* h, int ncols, int64_t nsamples, double alpha, int max_iter,
            double* x, double* info);

/* The reference's DLARS solver (contrib/dlars/src/dlars.C; chimes_lsq.py
 * --algorithm dlars | dlasso, src/chimes_lsq.py:714-790) on the normal equations:
 * LARS (lasso = 0) or LASSO (lasso = 1) steps from x = 0, the variable named by
 * each step entering next, stopping at the first path vertex whose objective
 * 0.5 ||b - A x||^2 / nsamples + lambda ||x||_1 exceeds the previous vertex's by
 * more than 1e-10 and returning that vertex, as the reference's driver does.
 * btb = b^T b.  colsum (device, ncols; NULL = no normalisation) = A^T 1 and bsum
 * = sum of b select --normalize=y: columns centred and scaled to unit norm, b
 * centred, coefficients returned unscaled (the fit's predictions are then
 * A x - (colsum / nsamples) . x + bsum / nsamples).  info (may be NULL):
 * iterations, active variables, objective of the previous vertex. */
int cg_dlars(cg_session* s, const double* G, const double* h, int ncols, int64_t nsamples, double btb, double lambda,
             int lasso, const double* colsum, double bsum, int max_iter, double* x, double* info);

/* cg_dlars with the reference DLARS driver's stopping and restart options
 * (contrib/dlars/src/dlars.C:96-100, 356-420, DLARS::print_restart / restart
 * :1543-2221): max_iter = --iterations; max_norm (> 0; 0 = none) = --max_norm: the
 * walk stops once the L1 norm of the coefficients after a step exceeds it and returns
 * the vertex before that step; restart_out (NULL = none) receives the walk's state
 * every ten iterations (iteration count, objective, coefficients, active set in entry
 * order, excluded variables, the variable named to enter next) and restart_in (NULL
 * = none) resumes a walk from such a file -- the active-set Cholesky factor is rebuilt
 * from G, so a resumed walk follows the uninterrupted one to rounding.  The file is
 * this library's text format, not the reference's restart.txt.  With colsum the
 * coefficients of the file are those of the normalised problem, as in the reference. */
int cg_dlars_ex(cg_session* s, const double* G, const double* h, int ncols, int64_t nsamples, double btb,
                double lambda, int lasso, const double* colsum, double bsum, int max_iter, double max_norm,
                const char* restart_in, const char* restart_out, double* x, double* info);

/* Work counters of the last assembly: accepted 2-body pairs, triplets, quadruplets,
 * and (cluster, allowed-power) evaluations of the 3- and 4-body terms. */
int cg_session_last_counts(const cg_session* s, int64_t* pairs, int64_t* triplets, int64_t* quads,
                           int64_t* evals3, int64_t* evals4);

/* Number of CUDA kernels the last assembly launched. */
int cg_session_last_launches(const cg_session* s, int64_t* launches);

/* Per-stage GPU time: with profiling on, the session records CUDA events around each
 * stage of every assembly (on its own stream) and around each row block's copy to the
 * host in the streamed calls (stage "host_copies").  cg_session_stage_times waits for
 * them and returns accumulated milliseconds and call counts for the CG_NSTAGES stages
 * named by cg_stage_name; cg_session_profile(s, 1) also clears the totals. */
#define CG_NSTAGES 18
int cg_session_profile(cg_session* s, int enable);
int cg_session_stage_times(cg_session* s, double* ms, int64_t* calls);
const char* cg_stage_name(int stage);

/* Message of the calling thread's last failure ("" if none). */
/* ---------------------------------------------------------------- MD force
 * The force-field evaluation of chimes_md for a batch of configurations:
 * ZCalc (src/functions.C:815-891) with Cheby::Force_all / Force_3B / Force_4B
 * (src/Cheby.C:1731-2675).  The coefficients are a fitted vector x with one value
 * per A column (the order of params.txt's coefficients), and the basis, cut-offs and
 * cluster map come from the model, as chimes_md takes them from params.txt. */
#define CG_MD_ENERGY_OFFSETS 1   /* add x's per-atom-type energy offsets to the energy */

/* Store the coefficients on the session's GPU.  precision: CG_FP64 (plain) or
 * CG_FP32 (cluster contraction in FP32, geometry and accumulation in FP64).
 * penalty_dist / penalty_scale: the 2-body penalty below s_min + dist (chimes_md
 * defaults 0.01 and 1.0e4, src/chimes_md.C:1747-1748). */
int cg_md_setup(cg_session* s, const double* x, int nx, int precision, int flags, double penalty_dist,
                double penalty_scale);

/* Forces (kcal/mol/A, 3 per atom in frame order; SYSTEM.ACCEL before the
 * division by mass) and 11 scalars per frame: potential energy (kcal/mol), the
 * pressure term PRESSURE_XYZ / (3V) and the 3x3 virial tensor / V (row-major,
 * kcal/mol/A^3, PRESSURE_TENSORS_XYZ_ALL).  cg_md_force takes host frames and
 * host outputs (copies included); cg_md_force_device works on uploaded frames and
 * device outputs. */
int cg_md_force(cg_session* s, const cg_frames* fr, double* forces, double* scalars);
int cg_md_force_device(cg_session* s, const cg_dframes* d, double* forces, double* scalars);

/* nsteps velocity-Verlet NVE steps of every uploaded frame (chimes_md with
 * CONSRNT NVE: UPDATE_COORDS, UPDATE_VELOCS_HALF_1 / _2, src/ClassDefs.C:870-1157).
 * mass: host, one per atom type (amu); dt_fs: time step in fs; velocities
 * (device, A per internal time unit of 48.888 fs, advanced in place) and the
 * positions of d are advanced; forces (device) holds the last step's forces.
 * scalars_steps ((nsteps+1) * nframes * 11) and ke_steps ((nsteps+1) * nframes,
 * kinetic energy) are device arrays receiving steps 0..nsteps, or NULL. */
int cg_md_nve(cg_session* s, cg_dframes* d, const double* mass, double dt_fs, int nsteps, double* velocities,
              double* forces, double* scalars_steps, double* ke_steps);

/* The same steps under a thermostat (chimes_md CONSRNT, src/ClassDefs.C:525-1460):
 * CG_NVT_MTK = NVT-MTK HOOVER tau (a Nose-Hoover thermostat integrated as Martyna,
 * Tobias and Klein, with the reference's 10-step velocity iteration), CG_NVT_BEREND
 * = NVT-BEREND tau (Berendsen velocity rescaling).  temperature in K, tau in fs;
 * every frame is its own system (N_DOF = 3N - 3).  conserved_steps
 * ((nsteps+1) * nframes, device, may be NULL) receives the thermostat's part of the
 * conserved quantity (CONSERVED_QUANT: Q zeta^2 / 2 + N_DOF kB T s; 0 for
 * Berendsen): the run's Econs = kinetic + potential + this term. */
enum { CG_NVT_MTK = 1, CG_NVT_BEREND = 2, CG_NVT_SCALE = 6 };
/* CG_NVT_SCALE = `CONSRNT NVT-SCALE n`: every n-th step the velocities are scaled by
 * sqrt(T / mean temperature of the last n steps) (CONSTRAINT::SCALE_VELOCITIES,
 * src/ClassDefs.C:1447-1469); tau_fs carries n. */

/* Fixed charges (FITCOUL false with non-zero ATMCHRG): subtract every frame's Ewald
 * Coulomb forces from its force labels on the session's GPU (SubtractEwaldForces,
 * src/Ewald.C:827-845, as process_frame does, src/chimes_lsq.C:800-801), with the
 * Ewald parameters of the batch's first frame.  A no-op for other models; call it
 * once on the batch cg_frames_read returned, before reading its labels. */
int cg_frames_subtract_coulomb(cg_session* s, cg_frames* fr);
int cg_md_nvt(cg_session* s, cg_dframes* d, const double* mass, double dt_fs, int nsteps, int style,
              double temperature, double tau_fs, double* velocities, double* forces, double* scalars_steps,
              double* ke_steps, double* conserved_steps);

/* NPT runs on uploaded frames (orthorhombic cells; the cells on the device change
 * with the run): CG_NPT_BEREND = `CONSRNT NPT-BEREND tau tau_baro` (Berendsen
 * velocity and isotropic position/cell scaling), CG_NPT_BEREND_ANISO = per-axis cell
 * scaling from the pressure tensor's diagonal, CG_NPT_MTK = `NPT-MTK HOOVER tau
 * tau_baro` (Martyna-Tobias-Klein thermostat and barostat with the reference's
 * 10-step velocity iteration).  Replaces CONSTRAINT::UPDATE_COORDS /
 * UPDATE_VELOCS_HALF_1 / _2 for those styles (src/ClassDefs.C:867-1424).
 * pressure in GPa (PRESSUR), time constants in fs; conserved_steps as cg_md_nvt
 * (NPT-MTK: thermostat and barostat energies + P V; 0 for Berendsen);
 * volume_steps ((nsteps+1) * nframes, device, may be NULL) receives each frame's
 * cell volume after each step. */
enum { CG_NPT_BEREND = 3, CG_NPT_BEREND_ANISO = 4, CG_NPT_MTK = 5 };
int cg_md_npt(cg_session* s, cg_dframes* d, const double* mass, double dt_fs, int nsteps, int style,
              double temperature, double tau_fs, double pressure_gpa, double tau_baro_fs, double* velocities,
              double* forces, double* scalars_steps, double* ke_steps, double* conserved_steps,
              double* volume_steps);

/* Finite-difference configurational pressure (what = 0: one PRESSURE_XYZ per frame,
 * PRSCALC NUMERICAL) or stress tensor (what = 1: nine PRESSURE_TENSORS_XYZ_ALL values
 * per frame, STRSCALC NUMERICAL) of host frames with the session's MD coefficients:
 * -dU/dV from cells scaled by 1 +- 1e-4, and (U(I - e E_ij) - U(I + e E_ij)) / (2 e V)
 * (numerical_pressure / numerical_stress_all, src/functions.C:402-628), every strained
 * replica of every frame evaluated in one batched force call. */
int cg_md_numerical(cg_session* s, const cg_frames* fr, int what, double* out);

/* ---- MD output files (host arrays; xyz in A, velocities and accelerations in the
 * MD's internal units as cg_md_* use them, cell = ax ay az bx by bz cx cy cz).
 * One trajectory frame in the format of `# TRAJEXT #` GEN / XYZ / LAMMPSTRJ
 * (WRITE_TRAJ::PRINT_FRAME_*, src/io_styles.C:322-423); frame_index 0 starts the
 * file, later frames append with the number format the reference's stream has by
 * then.  step is the MD step (printed as step + 1), temperature in K (GEN header),
 * wrap = `# WRPCRDS #`. */
enum { CG_TRAJ_GEN = 1, CG_TRAJ_XYZ = 2, CG_TRAJ_LAMMPSTRJ = 3 };
int cg_md_write_traj(const cg_model* m, int format, const char* path, int frame_index, int step, double dt_fs,
                     double temperature, int wrap, int natoms, const int* types, const double* xyz,
                     const double* velocities, const double* cell);

/* output.xyz of a run (write_xyzv, src/chimes_md.C:1207-1296, restart false). */
int cg_md_write_xyzv(const cg_model* m, const char* path, int natoms, const int* types, const double* xyz,
                     const double* velocities, const double* cell, int wrap);

/* restart.xyzv of frame `frame` after the session's last MD run: positions,
 * velocities, accelerations, step + 1, the neighbour padding, CONSTRAINT's 29 values
 * (CONSTRAINT::WRITE, from the run's thermostat / barostat state) and THERMO_AVG's 7
 * sums (avg7, may be NULL for zeros). */
int cg_md_write_restart(cg_session* s, int frame, const char* path, int natoms, const int* types, const double* xyz,
                        const double* velocities, const double* accel, const double* cell, int step,
                        double rcut_padding, const double* avg7, int wrap);

/* Read a restart.xyzv (read_restart_params, src/chimes_md.C:1298-1400): natoms must
 * match the file; constraint29 / avg7 receive its CONSTRAINT and THERMO_AVG blocks. */
int cg_md_read_restart(const cg_model* m, const char* path, int natoms, int* types, double* xyz,
                       double* velocities, double* accel, double* cell, int* step, double* rcut_padding,
                       double* constraint29, double* avg7);

/* Initial velocities of one system (internal units, [natoms][3]; mass per atom, amu):
 * generate != 0 draws them as `# VELINIT # GEN` does (C rand() seeded with `seed`,
 * Box-Muller, T in K), generate = 0 keeps v as read; either way the centre-of-mass
 * velocity is then removed (CONSTRAINT::INIT_VEL / CHECK_VEL, src/ClassDefs.C:617-788). */
int cg_md_velocities(int natoms, const double* mass, int generate, int seed, double temperature, double* v);

/* The session's next cg_md_nvt / cg_md_npt run starts each of its nframes frames
 * from these CONSTRAINT values (nframes x 29, as cg_md_read_restart returns them). */
int cg_md_resume(cg_session* s, int nframes, const double* constraint29);

/* Continuous-batching MD serving (no counterpart in the reference, whose chimes_md
 * runs one system).  Each request runs nsteps velocity-Verlet NVE steps (step 0
 * evaluates forces only, as chimes_md's first step) from its own positions and
 * velocities; it is admitted once its arrival time (seconds after the call starts)
 * has passed and the batch has room -- at most max_batch_atoms atoms and
 * max_batch_frames requests, and device memory within hbm_budget_bytes: the two
 * serving arenas (fixed for these capacities) plus, per admitted request, its atoms
 * times the list bytes per atom (cg_md_serve_memory; the lists' measured allocation
 * after every build replaces the prior) -- and every batched step advances all
 * admitted requests together; a request leaves the batch as soon as it finishes and
 * its final positions are copied to xyz_out.  A budget below the arenas, or a request
 * that cannot fit even alone, is refused (status 1 before any step, status 4 if the
 * measured list size rules it out later) instead of waiting forever.
 * results[r]: admission / finish times (seconds), sum and maximum of its step times
 * (ms), bytes reserved for it at admission.  step_ms (may be NULL): nreq *
 * max(nsteps) wall times (ms) of the batched step that advanced request r at step s.
 * *batch_steps: number of batched steps. */
typedef struct {
    int natoms, nsteps;
    double arrival;
    const int* types;
    const double* xyz;
    const double* cell;
    const double* v;
    double* xyz_out;
} cg_md_request;
typedef struct {
    double admitted, finished, step_ms_sum, step_ms_max, reserved_bytes;
} cg_md_result;
int cg_md_serve(cg_session* s, int nreq, const cg_md_request* req, const double* mass, double dt_fs,
                double hbm_budget_bytes, int64_t max_batch_atoms, int max_batch_frames, cg_md_result* results,
                double* step_ms, int64_t* batch_steps);

/* Live form of cg_md_serve (no counterpart in the reference): a thread of the library
 * runs the same batching loop on the session's GPU while the caller's threads submit
 * requests as they arrive and collect results, so a request submitted while others
 * are on the GPU joins the next batched step once the batch has room.  The session
 * belongs to the server until cg_md_server_stop (make no other call on it meanwhile).
 * Capacities and hbm_budget_bytes as in cg_md_serve; mass: one per atom type (amu). */
typedef struct cg_md_server cg_md_server;
int cg_md_server_start(cg_session* s, const double* mass, double dt_fs, double hbm_budget_bytes,
                       int64_t max_batch_atoms, int max_batch_frames, cg_md_server** out);
/* Queue one request (arrival = now: req->arrival and req->xyz_out are not read); its
 * inputs are copied before the call returns.  *ticket identifies it in
 * cg_md_server_poll.  Status 1 / 2 for a request that can never run: bad input, more
 * atoms than max_batch_atoms, more device memory than hbm_budget_bytes alone. */
int cg_md_server_submit(cg_md_server* srv, const cg_md_request* req, int64_t* ticket);
/* Status of a ticket: 0 once the request finished (result and, when xyz_out is not
 * NULL, its final positions, 3 per atom), CG_PENDING while it waits or runs (wait = 0),
 * or, with wait != 0, blocks until it finishes.  A failure of the serving loop (status
 * 3 or 4) is returned by every later poll and by cg_md_server_stop. */
#define CG_PENDING 5
int cg_md_server_poll(cg_md_server* srv, int64_t ticket, int wait, cg_md_result* result, double* xyz_out);
/* Stop taking requests, finish every queued and running one, end the thread and free
 * the server (also when a status is returned).  *batch_steps (may be NULL): batched
 * steps run. */
int cg_md_server_stop(cg_md_server* srv, int64_t* batch_steps);

/* Device memory of cg_md_serve for these capacities: arena_bytes = the two serving
 * arenas, bytes_per_atom = what an admitted request reserves per atom (the session's
 * last measured list size, or the prior before its first serving run).  Either output
 * may be NULL. */
int cg_md_serve_memory(cg_session* s, int64_t max_batch_atoms, int max_batch_frames, double* arena_bytes,
                       double* bytes_per_atom);

/* Device pointer to the positions of uploaded frames (3 per atom), and a copy of
 * them into host memory. */
int cg_dframes_positions(const cg_dframes* d, double** xyz, int64_t* natoms);
int cg_dframes_read_positions(const cg_dframes* d, double* xyz_host);

/* Pairs, triplets, quadruplets and kernel launches of the last MD force call. */
int cg_md_last_counts(const cg_session* s, int64_t* pairs, int64_t* triplets, int64_t* quads, int64_t* launches);

/* ---------------------------------------------------------------- batched fit
 * Thousands of frames in row blocks (uploaded with cg_frames_upload), each block
 * assembled into the caller's A buffer (a_precision, lda >= columns, rows >= the
 * largest block) and folded into G, h with the split-BF16 tensor-core Gram
 * (caller zeroes G and h; labels[k]: block k's b, device).  Create runs one sizing
 * pass per block (which also assembles it), then captures every block's launches
 * -- assembly and Gram, no host synchronisation -- as one CUDA graph; launch
 * replays the whole fit with one cudaGraphLaunch.  No counterpart in the reference
 * (its frames are processed one at a time, src/chimes_lsq.C:292-328). */
typedef struct cg_batch_fit cg_batch_fit;
int cg_batch_fit_create(cg_session* s, int nblocks, cg_dframes* const* blocks, const double* const* labels,
                        int a_precision, void* A, int64_t lda, double* G, double* h, cg_batch_fit** out);
int cg_batch_fit_launch(cg_session* s, cg_batch_fit* b);
int cg_batch_fit_nodes(const cg_batch_fit* b, int64_t* nodes);
void cg_batch_fit_free(cg_batch_fit* b);

/* Tunable launch parameters of a session (chosen by the autotuner,
 * chimes_lsq-myllfork_gb300/autotune.py): "gram_ctas_per_sm" (CTAs per SM the
 * tensor-core Gram aims for when it slices K; default 4); "md_skin_milli" (the
 * neighbour-list skin of cg_md_nve / cg_md_serve in 1e-3 A, default 500; 0 =
 * enumerate every step; lists are rebuilt when an atom has moved half the skin);
 * "gram_rows_per_launch" (rows of A summed in FP32 per tensor-core Gram launch before
 * they are added into the FP64 G; 0 = about 1 GiB of BF16 planes -- longer runs are
 * faster but their FP32 sums lose accuracy, which costs refinement passes);
 * "refine_cache_mb" (device memory the streamed refinement may fill with FP64 row
 * blocks kept between passes, in MiB; -1 = what is free beyond a margin, the
 * default; 0 = assemble every block on every pass); "force_range" (the many-body
 * force rows by the range form, each thread summing a contiguous range of a cluster
 * type's powers per column: 1, the default, in FP64 and, in FP32, where a type has
 * more than 512 allowed powers; 2 always; 0 never -- one accumulator per power, summed
 * per column in shared memory); "host_staging" (the pinned host buffers of cg_assemble_stream: 1, the
 * default, cudaMallocHost; 0, 512 MiB-aligned memory advised for transparent huge
 * pages and registered with CUDA); "force4_threads" (threads per CTA of the 4-body
 * force-row kernel when the
 * range form is not used, 512 or 1024); "cholesky_tensor_updates" (1, the
 * default: the blocked Cholesky's trailing updates from exact BF16 digit products on
 * the tensor cores, FP64-accurate; 0: the FP64 SYRK). */
int cg_session_tune(cg_session* s, const char* key, int value);

const char* cg_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* CHIMES_GB300_H */
