// Host-side model of a ChIMES-lsq fit: the fm_setup.in controls, the pair and
// cluster (triplet / quadruplet) topology with its permutation-invariant
// coefficient map, and the per-frame geometry read from .xyzf trajectories.
//
// This mirrors the reference's host setup so that the GPU kernels consume the
// same tables the reference builds:
//   INPUT::PARSE_INFILE_LSQ            src/input.C:172-225
//   CLUSTER::build / store_permutations src/Cluster.C:27-366
//   CLUSTER_LIST::build_pairs(_loop)    src/Cluster.C:1245-1484
//   CLUSTER::map_indices_int            src/Cluster.C:1768-1878
//   FRAME::READ_XYZF                    src/ClassDefs.C:2411-2683
//   BOX::UPDATE_CELL                    src/ClassDefs.C:1940-1971
#pragma once

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace cg {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

enum ChebTrans { TRANS_MORSE = 0, TRANS_INVRSE_R = 1, TRANS_NONE = 2 };
enum ChebFix { FIX_SMOOTH = 0, FIX_ZERO_DERIV = 1, FIX_CONSTANT_DERIV = 2 };
enum FcutKind { FCUT_CUBIC = 0, FCUT_TERSOFF = 1 };

struct PairType {
    int pairidx = 0;
    std::string atm1, atm2, prpr;
    int t1 = 0, t2 = 0;
    double chg1 = 0, chg2 = 0, mass1 = 0, mass2 = 0;
    std::string chrgsgn;
    double smin = 0.8, smax = 5.0, lambda = 0.0;
    double xmin = 0, xmax = 0, xavg = 0, xdiff = 0;
    double range_low = -1, range_high = 1;
    int snum = 0, snum3 = 0, snum4 = 0;
    int trans = TRANS_NONE;
    int col = 0;                      // first A column of its 2-body block; -1 when HIERARC excludes it
};

struct ClusterType {
    int index = 0, natoms = 0, npairs = 0;
    std::vector<std::string> atom_names, pair_names;
    std::vector<int> atom_indices;
    bool excluded = false, special_smax = false, special_smin = false;
    std::vector<double> smax, smin, xmin, xmax, xavg, xdiff;
    std::vector<std::vector<int>> allowed_powers, unique_powers;
    std::map<std::vector<int>, int> allowed_map;
    std::vector<int> equiv_indices, param_indices, power_count;
    int n_true = 0, n_allowed = 0;
};

struct ClusterList {
    int natoms = 0, npairs = 0, nclusters = 0;
    std::vector<ClusterType> vec;
    std::map<std::string, int> map;
    std::map<int, std::string> map_reverse;
    std::vector<int> int_map;                       // make_id_int(types) -> type index or -1
    std::vector<std::vector<int>> pair_indices;     // make_id_int(types) -> edge->slot map
    std::vector<int> int_map_reverse;
    std::vector<std::vector<std::string>> exclude;
    std::vector<std::string> smax_input, smin_input;
    double max_cutoff = 0.0;
};

struct Controls {
    std::vector<std::string> infile;
    std::vector<int> infile_frames;
    std::vector<std::string> force_flags, stress_flags, energy_flags;
    bool wrap = false;
    int nframes = 0, nlayers = 0;
    bool fit_coul = false, fit_stress = false, fit_stress_all = false, fit_ener = false;
    int nstress = -1, nener = -1;
    std::string ff_type;
    int cheby_order = 0, cheby3 = 0, cheby4 = 0;
    bool use3 = false, use4 = false;
    double range_low = -1, range_high = 1;
    int trans = TRANS_NONE;
    int fix = FIX_SMOOTH;
    double smooth = 0.01;
    bool use_neigh = true;
    bool force_small = false;
    int skip_frames = 0;
    int natmtyp = 0;
    std::string fcut_line = "CUBIC";
    int fcut = FCUT_CUBIC;
    double fcut_offset = 0.0;
    bool hierarchical = false, split_files = false;
    bool use_partial_charges = false;
};

// One CHARGE CONSTRAINTS line (src/input.C:1148-1200): sum_k value[k] * (q q)_pair[k]
// = force, appended to the fit as one row after all frames.
struct ChargeConstraint {
    std::vector<int> pair;
    std::vector<double> value;
    double force = 0.0;
};

struct Model {
    std::string dir;   // directory of fm_setup.in (trajectory paths are relative to it)
    Controls ctl;
    std::vector<PairType> pairs;
    std::map<std::string, int> pair_map;
    std::vector<int> int_pair_map;
    std::vector<std::string> atom_types;   // TYPEIDX order
    std::vector<int> atom_type_idx;
    ClusterList trips, quads;
    int tot_snum = 0, num3 = 0, num4 = 0, tot_short = 0, tot_all = 0;
    int ncoul = 0;                                   // FITCOUL: one q_i q_j column per pair type
    // HIERARC: atom types whose energy-offset column and pair types whose 2-body
    // columns the A matrix leaves out (EXCLUDE 1B / 2B INTERACTION, in input order)
    std::vector<int> excl1b, excl2b;
    std::vector<int> ener_col;                       // energy-offset column of each type (-1 excluded)
    std::vector<ChargeConstraint> charge_constraints;
    double max_cutoff_2b = 0, max_cutoff_3b = 0, max_cutoff_4b = 0;
    double deriv_const = 1.0;
};

// Parse fm_setup.in and build every table the design-matrix path needs.
Model load_model(const std::string& fm_setup_path);

// make_id_int: sum_i (type_i+1) * 10^i  (src/Cluster.C:1227-1237)
int make_id_int(const int* types, int n);

// Text writers for params.header and ff_groups.map (src/chimes_lsq.C:562-716).
std::string params_header_text(const Model& m);
std::string ff_groups_map_text(const Model& m);

// params.txt (the force field file written by chimes_lsq.py, src/chimes_lsq.py:284-675)
// for coefficients x (tot_all values): `preamble` is the "!"-comment block that the
// solver prints first; the rest follows params.header, the coefficient blocks and
// ff_groups.map exactly.
std::string params_txt_text(const Model& m, const double* x, int nx, const std::string& preamble);

// The charge-constraint rows of a FITCOUL fit (A_MAT::PRINT_CONSTRAINTS
// src/A_Matrix.C:569-625): row i is zero in the short-range columns and holds the
// constraint's value of each pair type in the charge columns; b[i] = its force.
// A is row-major with lda >= tot_all; writes charge_constraints.size() rows.
void constraint_rows(const Model& m, double* A, int64_t lda, double* b);

// Ewald parameters of one frame (optimal_ewald_params src/Ewald.C:428-475, with
// the accuracy 1e-6 of ZCalc_Ewald_Deriv): splitting alpha, real-space cut-off and
// integer k cut-off.
struct EwaldParams { double alpha = 0, rc = 0; int kmax = 0; };

// ---------------------------------------------------------------- frames

struct Box {
    bool is_ortho = true;
    double ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0, cx = 0, cy = 0, cz = 0;
    double hmat[9] = {0}, invr[9] = {0};
    double latcon_a = 0, latcon_b = 0, latcon_c = 0, alpha = 0, beta = 0, gamma = 0;
    double lx = 0, ly = 0, lz = 0, xy = 0, xz = 0, yz = 0;
    double xlo = 0, ylo = 0, zlo = 0, xhi = 0, yhi = 0, zhi = 0;
    double extent_x = 0, extent_y = 0, extent_z = 0, vol = 0;
    void update_cell();   // BOX::UPDATE_CELL
};

EwaldParams ewald_params(int natoms, const Box& box);

// BOX::WRAP_ATOM (src/ClassDefs.C:2064-2119): x moved into the primary cell.
void wrap_atom(const Box& b, double* x);

struct Frame {
    int natoms = 0;
    std::vector<int> type;            // index into Model::atom_types
    std::vector<double> xyz;          // 3*natoms, as read (wrapped when WRAPTRJ)
    std::vector<double> force;        // 3*natoms, kcal/mol/A
    Box box;
    double stress_diag[3] = {0, 0, 0};   // xx yy zz (GPa, as read)
    double stress_off[3] = {0, 0, 0};    // xy xz yz (GPa, as read)
    double energy = 0.0;
    int file = 0;                     // index of the TRJFILE the frame came from (label flags)
    int index = -1;                   // frame number in the trajectory (NSTRESS / NENER cut-offs)
    int rank = 0;                     // chimes_lsq rank that writes the frame (output order, SPLITFI)
};

// Frames that each of nprocs chimes_lsq ranks processes, in rank order: contiguous
// blocks (divide_atoms, src/functions.C:182-222) or, with SKPFRMS n >= 1, frame i on
// rank r when (i + r) % nprocs == 0 and ((i + r) / nprocs) % n == 0
// (src/chimes_lsq.C:305-317).  The ranks' files are concatenated in rank order.
std::vector<std::vector<int>> rank_frames(const Controls& c, int nprocs);

// Read the NFRAMES frames of the model's trajectory file(s) and keep the ones
// chimes_lsq on nprocs ranks would process, in the order of its output files.
std::vector<Frame> read_frames(const Model& m, int nprocs = 1);
// Read frames from one stream (exposed for tests and the C ABI).
std::vector<Frame> read_xyzf(const Model& m, const std::string& path, int nframes, int first_index,
                             Box& persistent_box);

// Per-frame row layout of the A matrix (src/A_Matrix.C:210-567).
struct RowLayout {
    int force_rows = 0, stress_rows = 0, energy_rows = 0;
    int total() const { return force_rows + stress_rows + energy_rows; }
};
RowLayout frame_rows(const Model& m, int frame_index, int natoms);

// Whether the frame uses the small-cell ("unordered", PERM_SCALE = 1/n!) neighbour
// convention (src/ClassDefs.C:44-67, 137-197).  The choice is sticky across frames
// in the reference, so the caller passes the state of the previous frame.
bool frame_is_small(const Model& m, const Box& box, bool previous_small);

}  // namespace cg
