// MD driver text files: trajectory frames, output.xyz and restart.xyzv, in the byte
// format of the reference's writers (WRITE_TRAJ src/io_styles.C:258-424; write_xyzv
// and read_restart_params src/chimes_md.C:1207-1400).
#include "mdio.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace cg {

namespace {

struct File {
    std::FILE* f = nullptr;
    File(const std::string& path, const char* mode) : f(std::fopen(path.c_str(), mode)) {
        if (!f) throw Error(2, "cannot open " + path + " for writing");
    }
    ~File() { if (f) std::fclose(f); }
};

Box box_of(const double* cell) {
    Box b;
    b.ax = cell[0]; b.ay = cell[1]; b.az = cell[2];
    b.bx = cell[3]; b.by = cell[4]; b.bz = cell[5];
    b.cx = cell[6]; b.cy = cell[7]; b.cz = cell[8];
    b.update_cell();
    return b;
}

// A double in the stream's current format: the default (%g, 6 significant digits)
// until the first coordinate line switched the stream to fixed with 5 decimals.
std::string num(double v, bool fixed5) {
    char b[64];
    std::snprintf(b, sizeof(b), fixed5 ? "%.5f" : "%g", v);
    return b;
}

const std::string& type_name(const Model& m, int t) {
    if (t < 0 || t >= (int)m.atom_types.size()) throw Error(1, "atom type index outside the model");
    return m.atom_types[t];
}

}  // namespace

void write_traj_frame(const Model& m, TrajFormat fmt, const std::string& path, int frame_index, int step,
                      double dt_fs, double temperature, bool wrap, const MdConfig& c) {
    if (frame_index < 0 || c.natoms < 0 || !c.xyz || !c.types || !c.cell) throw Error(1, "trajectory frame arrays");
    const bool later = frame_index > 0;
    File out(path, later ? "a" : "w");
    const Box b = box_of(c.cell);
    auto pos = [&](int i, double* x) {
        x[0] = c.xyz[3 * i]; x[1] = c.xyz[3 * i + 1]; x[2] = c.xyz[3 * i + 2];
        if (wrap) wrap_atom(b, x);
    };
    std::FILE* f = out.f;
    if (fmt == TRAJ_GEN) {   // PRINT_FRAME_GEN src/io_styles.C:322-359
        std::fprintf(f, "%5d S #Step %d Time %s (fs) Temp %s (k)\n", c.natoms, step + 1,
                     num((step + 1) * dt_fs, later).c_str(), num(temperature, later).c_str());
        for (const std::string& t : m.atom_types) std::fprintf(f, "%s ", t.c_str());
        std::fprintf(f, "\n");
        for (int i = 0; i < c.natoms; ++i) {
            double x[3];
            pos(i, x);
            std::fprintf(f, "%4d %2d %8.5f %8.5f %8.5f\n", i + 1, c.types[i] + 1, x[0], x[1], x[2]);
        }
        std::fprintf(f, "%8.5f %8.5f %8.5f\n", 0.0, 0.0, 0.0);
        std::fprintf(f, "%8.5f %8.5f %8.5f\n", b.ax, b.ay, b.az);
        std::fprintf(f, "%8.5f %8.5f %8.5f\n", b.bx, b.by, b.bz);
        std::fprintf(f, "%8.5f %8.5f %8.5f\n", b.cx, b.cy, b.cz);
    } else if (fmt == TRAJ_XYZ) {   // PRINT_FRAME_XYZ src/io_styles.C:361-385
        std::fprintf(f, "%d\n", c.natoms);
        if (b.is_ortho) {
            std::fprintf(f, "%s %s %s\n", num(b.ax, later).c_str(), num(b.by, later).c_str(), num(b.cz, later).c_str());
        } else {
            const double v[9] = {b.ax, b.ay, b.az, b.bx, b.by, b.bz, b.cx, b.cy, b.cz};
            std::fprintf(f, "NON_ORTHO");
            for (int k = 0; k < 9; ++k) std::fprintf(f, " %s", num(v[k], later).c_str());
            std::fprintf(f, "\n");
        }
        for (int i = 0; i < c.natoms; ++i) {
            double x[3];
            pos(i, x);
            std::fprintf(f, "%4s %15.5f %15.5f %15.5f\n", type_name(m, c.types[i]).c_str(), x[0], x[1], x[2]);
        }
    } else if (fmt == TRAJ_LAMMPSTRJ) {   // PRINT_FRAME_LAMMPSTRJ src/io_styles.C:387-423
        if (!c.v) throw Error(1, "the LAMMPSTRJ format needs velocities");
        std::fprintf(f, "ITEM: TIMESTEP\n%s\n", num((step + 1) * dt_fs, later).c_str());
        std::fprintf(f, "ITEM: NUMBER OF ATOMS\n%d\n", c.natoms);
        std::fprintf(f, "ITEM: BOX BOUNDS xy xz yz\n");
        std::fprintf(f, "0.0 %s %s\n", num(b.extent_x, later).c_str(), num(b.xy, later).c_str());
        std::fprintf(f, "0.0 %s %s\n", num(b.extent_y, later).c_str(), num(b.xz, later).c_str());
        std::fprintf(f, "0.0 %s %s\n", num(b.extent_z, later).c_str(), num(b.yz, later).c_str());
        std::fprintf(f, "ITEM: ATOMS id type element xu yu zu vx vy vz\n");
        for (int i = 0; i < c.natoms; ++i) {   // unwrapped coordinates
            const double* x = c.xyz + 3 * i;
            const double* v = c.v + 3 * i;
            std::fprintf(f, "%20d%4d%4s%15.5f%15.5f%15.5f%15.5f%15.5f%15.5f\n", i + 1, c.types[i] + 1,
                         type_name(m, c.types[i]).c_str(), x[0], x[1], x[2], v[0], v[1], v[2]);
        }
    } else {
        throw Error(1, "unknown trajectory format");
    }
}

void write_xyzv(const Model& m, const std::string& path, const MdConfig& c, bool wrap, const double* acc, int step,
                double rcut_padding, const double* constraint29, const double* avg7) {
    if (c.natoms < 0 || !c.xyz || !c.v || !c.types || !c.cell) throw Error(1, "configuration arrays");
    File out(path, "w");
    std::FILE* f = out.f;
    const Box b = box_of(c.cell);
    std::fprintf(f, "%5d\n", c.natoms);
    if (b.is_ortho) {
        std::fprintf(f, "%21.14e %21.14e %21.14e\n", b.ax, b.by, b.cz);
    } else {
        std::fprintf(f, "NON_ORTHO %21.14e %21.14e %21.14e %21.14e %21.14e %21.14e %21.14e %21.14e %21.14e\n", b.ax,
                     b.ay, b.az, b.bx, b.by, b.bz, b.cx, b.cy, b.cz);
    }
    for (int i = 0; i < c.natoms; ++i) {
        double x[3] = {c.xyz[3 * i], c.xyz[3 * i + 1], c.xyz[3 * i + 2]};
        if (wrap) wrap_atom(b, x);
        const double* v = c.v + 3 * i;
        std::fprintf(f, "%2s %21.14e %21.14e %21.14e    %21.14e %21.14e %21.14e ", type_name(m, c.types[i]).c_str(),
                     x[0], x[1], x[2], v[0], v[1], v[2]);
        if (acc) std::fprintf(f, "%21.14e %21.14e %21.14e\n", acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]);
        else std::fprintf(f, "\n");
    }
    if (acc) {   // the stream is in scientific / 14 digits by now
        std::fprintf(f, "%d\n%.14e\n", step, rcut_padding);
        for (int k = 0; k < RESTART_CONSTRAINT_FIELDS; ++k) std::fprintf(f, "%.14e\n", constraint29 ? constraint29[k] : 0.0);
        for (int k = 0; k < RESTART_AVG_FIELDS; ++k) std::fprintf(f, "%.14e\n", avg7 ? avg7[k] : 0.0);
    }
}

MdRestart read_restart(const Model& m, const std::string& path) {
    std::ifstream in(path);
    if (!in.is_open()) throw Error(2, "cannot open restart file " + path);
    MdRestart r;
    int n = 0;
    std::string line;
    if (!(in >> n) || n <= 0) throw Error(2, "restart file: bad atom count");
    std::getline(in, line);
    std::getline(in, line);
    std::istringstream cl(line);
    std::vector<std::string> tk;
    std::string w;
    while (cl >> w) tk.push_back(w);
    if (!tk.empty() && tk[0] == "NON_ORTHO") {
        if (tk.size() < 10) throw Error(2, "restart file: NON_ORTHO needs 9 cell components");
        for (int k = 0; k < 9; ++k) r.cell[k] = std::stod(tk[1 + k]);
    } else {
        if (tk.size() < 3) throw Error(2, "restart file: missing cell lengths");
        r.cell[0] = std::stod(tk[0]); r.cell[4] = std::stod(tk[1]); r.cell[8] = std::stod(tk[2]);
    }
    r.types.resize(n);
    r.xyz.resize(3 * (size_t)n);
    r.v.resize(3 * (size_t)n);
    r.acc.resize(3 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        std::string t;
        in >> t;
        size_t k = 0;
        for (; k < m.atom_types.size(); ++k) if (m.atom_types[k] == t) break;
        if (k == m.atom_types.size()) throw Error(2, "restart file: unknown atom type " + t);
        r.types[i] = (int)k;
        for (int q = 0; q < 3; ++q) in >> r.xyz[3 * i + q];
        for (int q = 0; q < 3; ++q) in >> r.v[3 * i + q];
        for (int q = 0; q < 3; ++q) in >> r.acc[3 * i + q];
    }
    if (!in) throw Error(2, "restart file: truncated atom lines");
    // the trailer as tokens through strtod: the reference writes members it never set,
    // which can be subnormal numbers that stream extraction rejects
    auto next = [&](const char* what) {
        std::string t;
        if (!(in >> t)) throw Error(2, std::string("restart file: truncated ") + what);
        return std::strtod(t.c_str(), nullptr);
    };
    r.step = (int)next("step line");
    r.rcut_padding = next("padding line");
    for (int k = 0; k < RESTART_CONSTRAINT_FIELDS; ++k) r.constraint[k] = next("constraint block");
    for (int k = 0; k < RESTART_AVG_FIELDS; ++k) r.avg[k] = next("average block");
    return r;
}

void md_velocities(int natoms, const double* mass, bool generate, int seed, double temperature, double* v) {
    if (natoms < 0 || (natoms > 0 && (!mass || !v))) throw Error(1, "velocity arrays");
    const double kb = 0.0019872067;   // src/functions.h:43
    if (generate) {
        std::srand((unsigned)seed);
        int counter = 0;
        for (int a = 0; a < natoms; ++a) {
            if (!(mass[a] > 0.0)) throw Error(1, "atom masses must be positive");
            const double sigma = std::sqrt(temperature * kb / mass[a]);
            for (int q = 0; q < 3; ++q, ++counter) {
                const double x1 = double(std::rand()) / double(RAND_MAX);
                const double x2 = double(std::rand()) / double(RAND_MAX);
                double y1 = std::sqrt(-2.0 * std::log(x1)) * std::cos(2.0 * M_PI * x2);
                double y2 = std::sqrt(-2.0 * std::log(x1)) * std::sin(2.0 * M_PI * x2);
                y1 *= sigma;
                y2 *= sigma;
                v[3 * a + q] = counter % 2 == 0 ? y2 : y1;
            }
        }
    }
    double p[3] = {0.0, 0.0, 0.0}, mt = 0.0;
    for (int a = 0; a < natoms; ++a) {
        for (int q = 0; q < 3; ++q) p[q] += mass[a] * v[3 * a + q];
        mt += mass[a];
    }
    if (mt > 0.0)
        for (int a = 0; a < natoms; ++a)
            for (int q = 0; q < 3; ++q) v[3 * a + q] -= p[q] / mt;
}

}  // namespace cg
