// Text files of the MD driver around the device force: trajectory frames (GEN, XYZ,
// LAMMPSTRJ), the final configuration output.xyz and the restart file restart.xyzv
// (WRITE_TRAJ src/io_styles.C:258-424, write_xyzv / read_restart_params
// src/chimes_md.C:1207-1400, CONSTRAINT::WRITE / READ src/ClassDefs.C:790-866,
// THERMO_AVG::WRITE src/ClassDefs.C:1627-1637).
#pragma once
#include <string>
#include <vector>

#include "model.h"

namespace cg {

enum TrajFormat { TRAJ_GEN = 1, TRAJ_XYZ = 2, TRAJ_LAMMPSTRJ = 3 };

// One configuration of an MD run (host arrays; velocities in the MD's internal units).
struct MdConfig {
    int natoms = 0;
    const int* types = nullptr;      // TYPEIDX order of the model
    const double* xyz = nullptr;     // [natoms][3]
    const double* v = nullptr;       // [natoms][3], may be null for GEN / XYZ
    const double* cell = nullptr;    // ax ay az bx by bz cx cy cz
};

// Append one frame (frame_index 0 starts the file).  The reference writes through
// one stream whose number format its coordinate lines switch to fixed / 5 decimals,
// so the header numbers of frame 0 print in the default format and later ones in
// that fixed format; frame_index reproduces this.
void write_traj_frame(const Model& m, TrajFormat fmt, const std::string& path, int frame_index, int step,
                      double dt_fs, double temperature, bool wrap, const MdConfig& c);

// CONSTRAINT's 29 restart values (WRITE order) and THERMO_AVG's 7 sums.
constexpr int RESTART_CONSTRAINT_FIELDS = 29;
constexpr int RESTART_AVG_FIELDS = 7;

// output.xyz (acc null) or restart.xyzv (acc set: accelerations and the trailer
// step + 1, neighbour padding, the constraint and average values).
void write_xyzv(const Model& m, const std::string& path, const MdConfig& c, bool wrap, const double* acc,
                int step, double rcut_padding, const double* constraint29, const double* avg7);

struct MdRestart {
    std::vector<int> types;
    std::vector<double> xyz, v, acc;
    double cell[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    int step = 0;                    // the file's step line (STEP + 1 of the run that wrote it)
    double rcut_padding = 0.0;
    double constraint[RESTART_CONSTRAINT_FIELDS] = {0};
    double avg[RESTART_AVG_FIELDS] = {0};
};
MdRestart read_restart(const Model& m, const std::string& path);

// Initial velocities (internal units) of natoms atoms with masses mass[i]:
// generate = VELINIT GEN (CONSTRAINT::INIT_VEL src/ClassDefs.C:617-713: C rand()
// seeded with `seed`, a Box-Muller pair per component whose sine and cosine halves
// alternate, sigma = sqrt(T kB / m)); then, as for read velocities, the mass-weighted
// centre-of-mass velocity is removed (CONSTRAINT::CHECK_VEL src/ClassDefs.C:715-788).
void md_velocities(int natoms, const double* mass, bool generate, int seed, double temperature, double* v);

}  // namespace cg
