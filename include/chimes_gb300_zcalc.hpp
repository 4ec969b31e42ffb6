/*
 * chimes_gb300_zcalc.hpp -- ZCalc / ZCalc_Deriv drop-ins over the C ABI of
 * chimes_gb300.h, for a chimes_md / chimes_lsq-style C++ driver.
 *
 * The reference's force and design-matrix calls take its own objects by reference:
 *   ZCalc(FRAME&, JOB_CONTROL&, vector<PAIR_FF>&, map<string,int>&, vector<int>&,
 *         CLUSTER_LIST&, CLUSTER_LIST&, NEIGHBORS&)                (src/functions.h:649)
 *   ZCalc_Deriv(JOB_CONTROL&, vector<PAIRS>&, CLUSTER_LIST&, CLUSTER_LIST&, FRAME&,
 *               A_MAT&, map<string,int>&, vector<int>&, NEIGHBORS&) (src/functions.h:632-633)
 * The functions below have the same parameters in the same order, as templates over
 * the caller's types, so a driver swaps the call without touching its arguments.
 * Ownership is the reference's: the caller owns every object; ZCalc writes
 * SYSTEM.ACCEL (forces before the division by mass), TOT_POT_ENER, PRESSURE_XYZ and
 * PRESSURE_TENSORS_XYZ_ALL (both already divided by the volume, as ZCalc leaves them,
 * src/functions.C:815-891) and zeroes PRESSURE_TENSORS_ALL; ZCalc_Deriv writes the
 * frame's A_MAT::FORCES[atom][column], STRESSES[column], FRAME_ENERGIES[column] and,
 * with FITCOUL, CHARGES[pair type][atom] (src/functions.C:755-804), which the caller
 * has sized as A_MAT::INITIALIZE does.
 *
 * What is read: SYSTEM.ATOMS, COORDS[a].X/Y/Z, ATOMTYPE_IDX[a] (the TYPEIDX order)
 * and BOXDIM.CELL_AX ... CELL_CZ.  The force-field arguments (JOB_CONTROL, the pair
 * and cluster lists, the maps, NEIGHBORS) are accepted for the signature and not
 * read: the bound Engine holds the same force field, parsed from the same
 * fm_setup.in (and, for ZCalc, the coefficients of the same params.txt), and the GPU
 * builds its own neighbour and cluster lists.  Errors, which the reference turns
 * into an exit of the process, throw std::runtime_error with the library's message.
 * Models with HIERARC 2-body exclusions are refused by ZCalc_Deriv (the excluded
 * columns exist in the reference's memory but not in this library's A).
 */
#ifndef CHIMES_GB300_ZCALC_HPP
#define CHIMES_GB300_ZCALC_HPP

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "chimes_gb300.h"

namespace chimes_gb300 {

inline void check(int rc, const char* what) {
    if (rc != 0) throw std::runtime_error(std::string(what) + ": " + cg_last_error());
}

// A force field on one GPU: the model of an fm_setup.in and a session.
class Engine {
   public:
    Engine(const char* fm_setup_path, int device = 0) {
        check(cg_model_load(fm_setup_path, &model_), "cg_model_load");
        if (cg_session_create(model_, device, &session_) != 0) {
            std::string m = cg_last_error();
            cg_model_free(model_);
            throw std::runtime_error("cg_session_create: " + m);
        }
        check(cg_model_columns(model_, &n2b_, &n3b_, &n4b_, nullptr, &ncols_), "cg_model_columns");
        check(cg_model_charge_columns(model_, &ncoul_, nullptr), "cg_model_charge_columns");
        check(cg_model_row_layout(model_, &stress_rows_, &energy_rows_), "cg_model_row_layout");
    }
    ~Engine() {
        cg_session_free(session_);
        cg_model_free(model_);
    }
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    // The MD coefficients from the text of a params.txt written for this model (as
    // chimes_md reads its PRMFILE); precision CG_FP64 or CG_FP32 (contraction form);
    // energy_offsets adds the per-atom-type offsets to the energy.
    void load_params(const std::string& params_txt, int precision = CG_FP64, bool energy_offsets = true,
                     double penalty_dist = 0.01, double penalty_scale = 1.0e4) {
        std::vector<double> x(ncols_);
        check(cg_model_params_read(model_, params_txt.c_str(), x.data(), ncols_), "cg_model_params_read");
        load_coefficients(x, precision, energy_offsets, penalty_dist, penalty_scale);
    }
    void load_coefficients(const std::vector<double>& x, int precision = CG_FP64, bool energy_offsets = true,
                           double penalty_dist = 0.01, double penalty_scale = 1.0e4) {
        check(cg_md_setup(session_, x.data(), (int)x.size(), precision, energy_offsets ? CG_MD_ENERGY_OFFSETS : 0,
                          penalty_dist, penalty_scale),
              "cg_md_setup");
    }

    cg_model* model() const { return model_; }
    cg_session* session() const { return session_; }
    int columns() const { return ncols_; }
    int short_range_columns() const { return n2b_ + n3b_ + n4b_; }
    int charge_columns() const { return ncoul_; }
    int stress_rows() const { return stress_rows_; }
    int energy_rows() const { return energy_rows_; }

    // One frame of n atoms (types in the TYPEIDX order, xyz in A, cell ax ay az bx by bz cx cy cz).
    cg_frames* frame(int n, const std::vector<int>& types, const std::vector<double>& xyz, const double* cell,
                     bool independent) const {
        cg_frames* fr = nullptr;
        check(cg_frames_create(model_, 1, &n, types.data(), xyz.data(), nullptr, cell, nullptr, nullptr, 0, &fr),
              "cg_frames_create");
        if (independent) check(cg_frames_independent(fr), "cg_frames_independent");
        return fr;
    }

   private:
    cg_model* model_ = nullptr;
    cg_session* session_ = nullptr;
    int n2b_ = 0, n3b_ = 0, n4b_ = 0, ncols_ = 0, ncoul_ = 0, stress_rows_ = 0, energy_rows_ = 0;
};

// The engine the drop-in calls use (set once by the driver, before the first call).
inline Engine*& bound_engine() {
    static Engine* e = nullptr;
    return e;
}
inline void bind(Engine* e) { bound_engine() = e; }
inline Engine& bound() {
    if (!bound_engine()) throw std::runtime_error("chimes_gb300: no Engine bound (call chimes_gb300::bind)");
    return *bound_engine();
}

namespace detail {
template <class FRAME>
void read_frame(const FRAME& S, std::vector<int>& types, std::vector<double>& xyz, double cell[9]) {
    const int n = S.ATOMS;
    types.resize(n);
    xyz.resize(3 * (size_t)n);
    for (int a = 0; a < n; ++a) {
        types[a] = S.ATOMTYPE_IDX[a];
        xyz[3 * a] = S.COORDS[a].X;
        xyz[3 * a + 1] = S.COORDS[a].Y;
        xyz[3 * a + 2] = S.COORDS[a].Z;
    }
    const double c[9] = {S.BOXDIM.CELL_AX, S.BOXDIM.CELL_AY, S.BOXDIM.CELL_AZ, S.BOXDIM.CELL_BX, S.BOXDIM.CELL_BY,
                         S.BOXDIM.CELL_BZ, S.BOXDIM.CELL_CX, S.BOXDIM.CELL_CY, S.BOXDIM.CELL_CZ};
    for (int k = 0; k < 9; ++k) cell[k] = c[k];
}
}  // namespace detail

// ZCalc (src/functions.h:649) on the bound engine's GPU.
template <class FRAME, class JOB_CONTROL, class PAIR_FF, class CLUSTER_LIST, class NEIGHBORS>
void ZCalc(FRAME& SYSTEM, JOB_CONTROL& CONTROLS, std::vector<PAIR_FF>& FF_2BODY, std::map<std::string, int>& PAIR_MAP,
           std::vector<int>& INT_PAIR_MAP, CLUSTER_LIST& TRIPS, CLUSTER_LIST& QUADS, NEIGHBORS& NEIGHBOR_LIST) {
    (void)CONTROLS; (void)FF_2BODY; (void)PAIR_MAP; (void)INT_PAIR_MAP; (void)TRIPS; (void)QUADS;
    (void)NEIGHBOR_LIST;
    Engine& e = bound();
    std::vector<int> types;
    std::vector<double> xyz;
    double cell[9];
    detail::read_frame(SYSTEM, types, xyz, cell);
    const int n = SYSTEM.ATOMS;
    cg_frames* fr = e.frame(n, types, xyz, cell, true);
    std::vector<double> F(3 * (size_t)n), sc(11);
    const int rc = cg_md_force(e.session(), fr, F.data(), sc.data());
    cg_frames_free(fr);
    check(rc, "cg_md_force");
    if ((int)SYSTEM.ACCEL.size() < n) SYSTEM.ACCEL.resize(n);
    for (int a = 0; a < n; ++a) {
        SYSTEM.ACCEL[a].X = F[3 * a];
        SYSTEM.ACCEL[a].Y = F[3 * a + 1];
        SYSTEM.ACCEL[a].Z = F[3 * a + 2];
    }
    SYSTEM.TOT_POT_ENER = sc[0];
    SYSTEM.PRESSURE_XYZ = sc[1];
    SYSTEM.PRESSURE_TENSORS_XYZ_ALL.resize(3);
    SYSTEM.PRESSURE_TENSORS_ALL.resize(3);
    for (int i = 0; i < 3; ++i) {
        SYSTEM.PRESSURE_TENSORS_XYZ_ALL[i].X = sc[2 + 3 * i];
        SYSTEM.PRESSURE_TENSORS_XYZ_ALL[i].Y = sc[3 + 3 * i];
        SYSTEM.PRESSURE_TENSORS_XYZ_ALL[i].Z = sc[4 + 3 * i];
        SYSTEM.PRESSURE_TENSORS_ALL[i].X = 0.0;
        SYSTEM.PRESSURE_TENSORS_ALL[i].Y = 0.0;
        SYSTEM.PRESSURE_TENSORS_ALL[i].Z = 0.0;
    }
}

// ZCalc_Deriv (src/functions.h:632-633) on the bound engine's GPU: one frame's A rows.
template <class JOB_CONTROL, class PAIRS, class CLUSTER_LIST, class FRAME, class A_MAT, class NEIGHBORS>
void ZCalc_Deriv(JOB_CONTROL& CONTROLS, std::vector<PAIRS>& FF_2BODY, CLUSTER_LIST& TRIPS, CLUSTER_LIST& QUADS,
                 FRAME& FRAME_SYSTEM, A_MAT& A_MATRIX, std::map<std::string, int>& PAIR_MAP,
                 std::vector<int>& INT_PAIR_MAP, NEIGHBORS& NEIGHBOR_LIST) {
    (void)CONTROLS; (void)FF_2BODY; (void)TRIPS; (void)QUADS; (void)PAIR_MAP; (void)INT_PAIR_MAP;
    (void)NEIGHBOR_LIST;
    Engine& e = bound();
    const int n = FRAME_SYSTEM.ATOMS, C = e.columns(), ns = e.short_range_columns();
    if ((int)A_MATRIX.FORCES.size() < n) throw std::runtime_error("ZCalc_Deriv: A_MAT::FORCES has fewer atoms");
    for (int a = 0; a < n; ++a)
        if ((int)A_MATRIX.FORCES[a].size() != ns)
            throw std::runtime_error("ZCalc_Deriv: A_MAT::FORCES[atom] is not sized to the short-range column count "
                                     "(HIERARC 2-body exclusions are not supported by this shim)");
    std::vector<int> types;
    std::vector<double> xyz;
    double cell[9];
    detail::read_frame(FRAME_SYSTEM, types, xyz, cell);
    cg_frames* fr = e.frame(n, types, xyz, cell, false);
    int64_t rows = 0;
    int rc = cg_frames_rows(fr, &rows, nullptr);
    std::vector<double> A;
    if (rc == 0) {
        A.resize((size_t)rows * C);
        rc = cg_assemble(e.session(), fr, CG_FP64, A.data(), C);
    }
    cg_frames_free(fr);
    check(rc, "cg_assemble");
    auto at = [&](int64_t r, int c) { return A[(size_t)r * C + c]; };
    for (int a = 0; a < n; ++a)
        for (int c = 0; c < ns; ++c) {
            A_MATRIX.FORCES[a][c].X = at(3 * a, c);
            A_MATRIX.FORCES[a][c].Y = at(3 * a + 1, c);
            A_MATRIX.FORCES[a][c].Z = at(3 * a + 2, c);
        }
    for (int i = 0; i < e.charge_columns() && i < (int)A_MATRIX.CHARGES.size(); ++i)
        for (int a = 0; a < n && a < (int)A_MATRIX.CHARGES[i].size(); ++a) {
            A_MATRIX.CHARGES[i][a].X = at(3 * a, ns + i);
            A_MATRIX.CHARGES[i][a].Y = at(3 * a + 1, ns + i);
            A_MATRIX.CHARGES[i][a].Z = at(3 * a + 2, ns + i);
        }
    const int64_t r0 = 3 * (int64_t)n;
    if (e.stress_rows() > 0 && (int)A_MATRIX.STRESSES.size() >= ns)
        for (int c = 0; c < ns; ++c) {
            if (e.stress_rows() == 3) {   // xx yy zz
                A_MATRIX.STRESSES[c].XX = at(r0, c);
                A_MATRIX.STRESSES[c].YY = at(r0 + 1, c);
                A_MATRIX.STRESSES[c].ZZ = at(r0 + 2, c);
            } else {                      // xx xy xz xy yy yz xz yz zz
                A_MATRIX.STRESSES[c].XX = at(r0, c);
                A_MATRIX.STRESSES[c].XY = at(r0 + 1, c);
                A_MATRIX.STRESSES[c].XZ = at(r0 + 2, c);
                A_MATRIX.STRESSES[c].YY = at(r0 + 4, c);
                A_MATRIX.STRESSES[c].YZ = at(r0 + 5, c);
                A_MATRIX.STRESSES[c].ZZ = at(r0 + 8, c);
            }
        }
    if (e.energy_rows() > 0 && (int)A_MATRIX.FRAME_ENERGIES.size() >= ns)
        for (int c = 0; c < ns; ++c) A_MATRIX.FRAME_ENERGIES[c] = at(r0 + e.stress_rows(), c);
}

}  // namespace chimes_gb300

#endif /* CHIMES_GB300_ZCALC_HPP */
