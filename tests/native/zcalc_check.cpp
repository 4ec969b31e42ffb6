// A chimes_md / chimes_lsq-style C++ caller of the ZCalc / ZCalc_Deriv drop-ins
// (include/chimes_gb300_zcalc.hpp).  The object types below carry only the members
// the drop-ins use, with the reference's names (src/functions.h, src/A_Matrix.h);
// a driver built on the reference's own classes compiles against the same calls.
//
//   zcalc_check MD_FM_SETUP MD_FRAME MD_COEF OUT_F LSQ_FM_SETUP LSQ_FRAME OUT_A
//
// Frame files: int32 natoms, int32 types[natoms], double xyz[3 natoms], double
// cell[9]; coefficient file: int32 n, double x[n].  OUT_F: ACCEL (3 per atom), then
// TOT_POT_ENER, PRESSURE_XYZ and the 9 PRESSURE_TENSORS_XYZ_ALL values.  OUT_A: the
// frame's rows rebuilt from A_MAT (force x, y, z per atom, then xx xy xz xy yy yz xz
// yz zz, then the energy row three times) over the short-range columns.
#include <cstdio>
#include <fstream>
#include <iterator>
#include <map>
#include <string>
#include <vector>

#include "chimes_gb300_zcalc.hpp"

struct XYZ { double X = 0, Y = 0, Z = 0; };
struct STENSOR { double XX = 0, YY = 0, ZZ = 0, XY = 0, XZ = 0, YZ = 0; };
struct BOX { double CELL_AX = 0, CELL_AY = 0, CELL_AZ = 0, CELL_BX = 0, CELL_BY = 0, CELL_BZ = 0,
             CELL_CX = 0, CELL_CY = 0, CELL_CZ = 0; };
struct FRAME {
    int ATOMS = 0;
    BOX BOXDIM;
    std::vector<int> ATOMTYPE_IDX;
    std::vector<XYZ> COORDS, ACCEL;
    double TOT_POT_ENER = 0, PRESSURE_XYZ = 0;
    std::vector<XYZ> PRESSURE_TENSORS_XYZ_ALL, PRESSURE_TENSORS_ALL;
};
struct A_MAT {
    std::vector<std::vector<XYZ> > FORCES;
    std::vector<STENSOR> STRESSES;
    std::vector<double> FRAME_ENERGIES;
    std::vector<std::vector<XYZ> > CHARGES;
};
struct JOB_CONTROL {};
struct PAIRS {};
struct PAIR_FF {};
struct CLUSTER_LIST {};
struct NEIGHBORS {};

static std::vector<char> slurp(const char* p) {
    std::ifstream f(p, std::ios::binary);
    return std::vector<char>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

static FRAME load_frame(const char* p) {
    const std::vector<char> b = slurp(p);
    FRAME S;
    S.ATOMS = *reinterpret_cast<const int*>(b.data());
    const int* t = reinterpret_cast<const int*>(b.data() + 4);
    const double* x = reinterpret_cast<const double*>(b.data() + 4 + 4 * (size_t)S.ATOMS);
    const double* c = x + 3 * (size_t)S.ATOMS;
    S.ATOMTYPE_IDX.assign(t, t + S.ATOMS);
    S.COORDS.resize(S.ATOMS);
    S.ACCEL.resize(S.ATOMS);
    for (int a = 0; a < S.ATOMS; ++a) { S.COORDS[a].X = x[3 * a]; S.COORDS[a].Y = x[3 * a + 1]; S.COORDS[a].Z = x[3 * a + 2]; }
    BOX& B = S.BOXDIM;
    B.CELL_AX = c[0]; B.CELL_AY = c[1]; B.CELL_AZ = c[2]; B.CELL_BX = c[3]; B.CELL_BY = c[4]; B.CELL_BZ = c[5];
    B.CELL_CX = c[6]; B.CELL_CY = c[7]; B.CELL_CZ = c[8];
    return S;
}

int main(int argc, char** argv) {
    if (argc != 8) {
        std::fprintf(stderr, "usage: zcalc_check MD_FM_SETUP MD_FRAME MD_COEF OUT_F LSQ_FM_SETUP LSQ_FRAME OUT_A\n");
        return 2;
    }
    try {
        JOB_CONTROL controls;
        std::map<std::string, int> pair_map;
        std::vector<int> int_pair_map;
        CLUSTER_LIST trips, quads;
        NEIGHBORS neigh;
        {   // MD force
            chimes_gb300::Engine md(argv[1]);
            const std::vector<char> cb = slurp(argv[3]);
            const int n = *reinterpret_cast<const int*>(cb.data());
            const double* x = reinterpret_cast<const double*>(cb.data() + 4);
            md.load_coefficients(std::vector<double>(x, x + n));
            chimes_gb300::bind(&md);
            FRAME S = load_frame(argv[2]);
            std::vector<PAIR_FF> ff(1);
            chimes_gb300::ZCalc(S, controls, ff, pair_map, int_pair_map, trips, quads, neigh);
            std::vector<double> out;
            for (const XYZ& a : S.ACCEL) { out.push_back(a.X); out.push_back(a.Y); out.push_back(a.Z); }
            out.push_back(S.TOT_POT_ENER);
            out.push_back(S.PRESSURE_XYZ);
            for (const XYZ& r : S.PRESSURE_TENSORS_XYZ_ALL) { out.push_back(r.X); out.push_back(r.Y); out.push_back(r.Z); }
            std::ofstream(argv[4], std::ios::binary).write(reinterpret_cast<const char*>(out.data()),
                                                           out.size() * sizeof(double));
        }
        {   // design-matrix rows of one frame
            chimes_gb300::Engine lsq(argv[5]);
            chimes_gb300::bind(&lsq);
            FRAME S = load_frame(argv[6]);
            const int ns = lsq.short_range_columns();
            A_MAT A;
            A.FORCES.assign(S.ATOMS, std::vector<XYZ>(ns));
            A.STRESSES.assign(ns, STENSOR());
            A.FRAME_ENERGIES.assign(ns, 0.0);
            std::vector<PAIRS> ff(1);
            chimes_gb300::ZCalc_Deriv(controls, ff, trips, quads, S, A, pair_map, int_pair_map, neigh);
            std::vector<double> out;
            for (int a = 0; a < S.ATOMS; ++a) {
                for (int c = 0; c < ns; ++c) out.push_back(A.FORCES[a][c].X);
                for (int c = 0; c < ns; ++c) out.push_back(A.FORCES[a][c].Y);
                for (int c = 0; c < ns; ++c) out.push_back(A.FORCES[a][c].Z);
            }
            double STENSOR::*comp[9] = {&STENSOR::XX, &STENSOR::XY, &STENSOR::XZ, &STENSOR::XY, &STENSOR::YY,
                                        &STENSOR::YZ, &STENSOR::XZ, &STENSOR::YZ, &STENSOR::ZZ};
            for (int r = 0; r < 9; ++r)
                for (int c = 0; c < ns; ++c) out.push_back(A.STRESSES[c].*comp[r]);
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < ns; ++c) out.push_back(A.FRAME_ENERGIES[c]);
            std::ofstream(argv[7], std::ios::binary).write(reinterpret_cast<const char*>(out.data()),
                                                           out.size() * sizeof(double));
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "zcalc_check: %s\n", e.what());
        return 1;
    }
    std::printf("zcalc_check: ok\n");
    return 0;
}
