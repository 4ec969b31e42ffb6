// Text files of the fit: A.txt / b.txt / b-labeled.txt / natoms.txt / dim.txt
// (A_MAT::PRINT_FRAME and CLEANUP_FILES, src/A_Matrix.C:210-720) and the
// coefficient reader of params.txt (the inverse of params_txt_text).
#include "textio.h"

#include <cstdio>
#include <algorithm>
#include <fstream>
#include <memory>
#include <sstream>
#include <vector>

namespace cg {

namespace {

struct Out {
    std::FILE* f = nullptr;
    explicit Out(const std::string& path) : f(std::fopen(path.c_str(), "w")) {
        if (!f) throw Error(2, "cannot open " + path + " for writing");
    }
    ~Out() { if (f) std::fclose(f); }
    void num(double v) { std::fprintf(f, "%.16e", v); }
    void lab(double v) { std::fprintf(f, "%g", v); }   // default ostream format (6 significant digits)
    void s(const char* t) { std::fputs(t, f); }
};

}  // namespace

// Row order and separators follow PRINT_FRAME: force rows "%.16e   " per column,
// b-labeled.txt values in the default stream format (%g),
// stress and energy rows "%.16e " per column; with energy fitting each row ends in
// " 0.0" per atom type (force / stress rows) or " <count of that type>" (energy rows).
// FITCOUL: force rows carry the charge columns after the short-range ones, and the
// charge-constraint rows follow the last frame ("0.0 " short-range, then the values).
// natoms.txt has the frame's atom count per row; dim.txt "columns rows".
// Frames of an emulated multi-rank run are written in rank order (the reference
// concatenates its per-rank files); with SPLITFI the A rows stay in A.%04d.txt per
// rank with data and dim.%04d.txt holds "columns first-row last-row total".
// A == nullptr writes the label files and dimensions only.
void write_lsq_files(const Model& m, const FrameBatch& fb, const double* A, int64_t lda, const std::string& dir,
                     bool with_constraints) {
    const int C = m.tot_short;
    const int nener = m.tot_all - m.tot_short - m.ncoul;
    const bool do_ener = nener > 0;
    const int nprocs = std::max(1, fb.nprocs);
    const bool split = m.ctl.split_files;
    auto rank_of = [&](int f) { return f < (int)fb.rank.size() ? fb.rank[f] : 0; };
    for (int f = 1; f < fb.nframes; ++f)
        if (rank_of(f) < rank_of(f - 1)) throw Error(1, "frames are not in rank order");
    const bool constraints = with_constraints && !m.charge_constraints.empty();
    // rows per rank; the constraint rows go to the first rank without data when the
    // files stay split, else to the last rank (A_MAT::PRINT_CONSTRAINTS :570-604)
    std::vector<int64_t> count(nprocs, 0);
    for (int f = 0; f < fb.nframes; ++f) count[rank_of(f)] += fb.row_ofs[f + 1] - fb.row_ofs[f];
    int print_rank = nprocs - 1;
    if (split)
        for (int r = 0; r < nprocs; ++r) if (count[r] == 0) { print_rank = r; break; }
    if (constraints) count[print_rank] += (int64_t)m.charge_constraints.size();
    Out fbv(dir + "/b.txt"), fbl(dir + "/b-labeled.txt"), fna(dir + "/natoms.txt");
    std::unique_ptr<Out> fa;
    if (A && !split) fa.reset(new Out(dir + "/A.txt"));
    auto flag = [&](const std::vector<std::string>& v, int f) -> const char* {   // INFILE_*_FLAGS[my_file]
        const int k = f < (int)fb.file.size() ? fb.file[f] : 0;
        return k < (int)v.size() ? v[k].c_str() : "";
    };
    int64_t total = 0;
    for (int r = 0; r < nprocs; ++r) total += count[r];
    int64_t start = 0;
    int f = 0;
    for (int r = 0; r < nprocs; ++r) {
        char name[64];
        if (A && split && count[r] > 0) {
            std::snprintf(name, sizeof(name), "/A.%04d.txt", r);
            fa.reset(new Out(dir + name));
        }
        for (; f < fb.nframes && rank_of(f) == r; ++f) {
            const int N = fb.natoms[f];
            const int64_t a0 = fb.atom_ofs[f];
            std::vector<int> natyp(m.ctl.natmtyp, 0);
            for (int a = 0; a < N; ++a) natyp[fb.type[a0 + a]]++;
            auto row_out = [&](int64_t r_, int ncols, const char* sep, bool energy) {
                if (fa) {
                    const double* Ar = A + r_ * lda;
                    for (int c = 0; c < ncols; ++c) { fa->num(Ar[c]); fa->s(sep); }
                    if (do_ener)
                        for (int t = 0; t < m.ctl.natmtyp; ++t) {
                            if (m.ener_col[t] < 0) continue;   // HIERARC EXCLUDE 1B
                            if (energy) std::fprintf(fa->f, " %d", natyp[t]);
                            else fa->s(" 0.0");
                        }
                    fa->s("\n");
                }
                std::fprintf(fna.f, "%d\n", N);
            };
            const int64_t r0 = fb.row_ofs[f];
            for (int a = 0; a < N; ++a) {
                for (int q = 0; q < 3; ++q) {
                    row_out(r0 + 3 * a + q, C + m.ncoul, "   ", false);   // + charge columns
                    const double bv = fb.b[r0 + 3 * a + q];
                    fbv.num(bv); fbv.s("\n");
                    fbl.s(flag(m.ctl.force_flags, f)); fbl.s(m.atom_types[fb.type[a0 + a]].c_str()); fbl.s(" ");
                    fbl.lab(bv); fbl.s("\n");
                }
            }
            const int srows = fb.stress_rows[f], erows = fb.energy_rows[f];
            static const char* l3[3] = {"s_xx ", "s_yy ", "s_zz "};
            static const char* l9[9] = {"s_xx ", "s_xy ", "s_xz ", "s_yx ", "s_yy ", "s_yz ", "s_zx ", "s_zy ", "s_zz "};
            for (int k = 0; k < srows; ++k) {
                const int64_t rr = r0 + 3 * N + k;
                row_out(rr, C, " ", false);
                fbv.num(fb.b[rr]); fbv.s("\n");
                fbl.s(flag(m.ctl.stress_flags, f)); fbl.s(srows == 3 ? l3[k] : l9[k]); fbl.lab(fb.b[rr]); fbl.s("\n");
            }
            for (int k = 0; k < erows; ++k) {
                const int64_t rr = r0 + 3 * N + srows + k;
                row_out(rr, C, " ", true);
                fbv.num(fb.b[rr]); fbv.s("\n");
                fbl.s(flag(m.ctl.energy_flags, f)); fbl.s("+1 "); fbl.lab(fb.b[rr]); fbl.s("\n");
            }
        }
        if (constraints && r == print_rank) {   // A_MAT::PRINT_CONSTRAINTS src/A_Matrix.C:606-623
            if (A && split && !fa) {
                std::snprintf(name, sizeof(name), "/A.%04d.txt", r);
                fa.reset(new Out(dir + name));
            }
            const int np = (int)m.pairs.size();
            for (const ChargeConstraint& cc : m.charge_constraints) {
                if (fa) {
                    for (int c = 0; c < C; ++c) fa->s("0.0 ");
                    for (int j = 0; j < np; ++j)
                        for (size_t k = 0; k < cc.pair.size(); ++k)
                            if (cc.pair[k] == j) { fa->num(cc.value[k]); fa->s(" "); }
                    fa->s("\n");
                }
                fbv.num(cc.force); fbv.s("\n");
            }
        }
        if (split) {
            fa.reset();
            if (count[r] > 0) {   // CLEANUP_FILES src/A_Matrix.C:681-704: columns, first row, last row, total
                std::snprintf(name, sizeof(name), "/dim.%04d.txt", r);
                Out fd(dir + name);
                std::fprintf(fd.f, "%d %lld %lld %lld\n", m.tot_all, (long long)start,
                             (long long)(start + count[r] - 1), (long long)total);
            }
        }
        start += count[r];
    }
    if (!split) {
        Out fd(dir + "/dim.txt");
        std::fprintf(fd.f, "%d %lld\n", m.tot_all, (long long)total);
    }
}

// Coefficients from params.txt text: the 2-body blocks ("%3d %21.13e" lines after
// "PAIRTYPE PARAMS:"), the cluster power lines (last field, param-index column) and
// the energy offsets, placed in A-column order (src/chimes_lsq.py:462-672).
std::vector<double> params_txt_coefficients(const Model& m, const std::string& text) {
    std::vector<double> x(m.tot_all, 0.0);
    std::vector<char> seen(m.tot_all, 0);
    std::istringstream in(text);
    std::string line;
    std::vector<std::string> lines;
    while (std::getline(in, line)) lines.push_back(line);
    auto toks = [](const std::string& l) {
        std::vector<std::string> t;
        std::istringstream ss(l);
        std::string w;
        while (ss >> w) t.push_back(w);
        return t;
    };
    const int snum = m.ctl.cheby_order;
    int section = 0, pair = -1, ctype = -1, base = 0, tpar = 0;
    const ClusterList* cl = nullptr;
    auto put = [&](int col, double v) {
        if (col < 0 || col >= m.tot_all) throw Error(2, "params.txt names a coefficient outside the model");
        x[col] = v;
        seen[col] = 1;
    };
    for (const std::string& l : lines) {
        const auto t = toks(l);
        if (t.empty() || t[0][0] == '!') continue;
        if (t[0] == "PAIRMAPS:" || t[0] == "ENDFILE") { section = 0; continue; }   // ff_groups.map echo
        if (t.size() >= 3 && t[2] == "PARAMS" && (t[0] == "PAIR" || t[0] == "TRIPLET" || t[0] == "QUADRUPLET")) {
            section = t[0] == "PAIR" ? 2 : (t[0] == "TRIPLET" ? 3 : 4);
            cl = section == 3 ? &m.trips : (section == 4 ? &m.quads : nullptr);
            base = section == 3 ? m.tot_snum : m.tot_snum + m.num3;
            ctype = -1;
            tpar = 0;
            continue;
        }
        if (section == 2 && t.size() >= 3 && t[0] == "PAIRTYPE" && t[1] == "PARAMS:") { pair = std::stoi(t[2]); continue; }
        if ((section == 3 || section == 4) && t[0].rfind(section == 3 ? "TRIPLETTYPE" : "QUADRUPLETYPE", 0) == 0) {
            if (ctype >= 0) tpar += cl->vec[ctype].n_true;
            ++ctype;
            continue;
        }
        if (t.size() >= 4 && t[0] == "ENERGY" && t[1] == "OFFSET") {
            const int ty = std::stoi(t[2]) - 1;   // HIERARC-excluded types print 0 and have no column
            if (ty < 0 || ty >= (int)m.ener_col.size()) throw Error(2, "params.txt names an unknown atom type");
            if (m.ener_col[ty] >= 0) put(m.tot_short + m.ncoul + m.ener_col[ty], std::stod(t[3]));
            continue;
        }
        if (section == 2 && pair >= 0 && m.ncoul > 0 && t.size() == 4 && t[1] == "x" && t[0].rfind("q_", 0) == 0) {
            put(m.tot_short + pair, std::stod(t[3]));   // charge product of the pair (FITCOUL)
            continue;
        }
        if (section == 2 && pair >= 0 && t.size() == 2 && snum > 0 && t[0].find_first_not_of("0123456789") == std::string::npos) {
            const int k = std::stoi(t[0]);
            if (pair >= (int)m.pairs.size()) throw Error(2, "params.txt names an unknown pair type");
            if (k < snum && m.pairs[pair].col >= 0) put(m.pairs[pair].col + k, std::stod(t[1]));
            continue;
        }
        if ((section == 3 || section == 4) && ctype >= 0 && ctype < (int)cl->vec.size()) {
            const int npw = section == 3 ? 3 : 6;
            if ((int)t.size() == npw + 4) {   // index, powers, equiv index, param index, value
                bool numeric = true;
                for (int k = 0; k < npw + 3 && numeric; ++k)
                    numeric = t[k].find_first_not_of("0123456789") == std::string::npos;
                if (numeric) put(base + tpar + std::stoi(t[npw + 2]), std::stod(t[npw + 3]));
            }
        }
    }
    for (int c = 0; c < m.tot_all; ++c)
        if (!seen[c]) throw Error(2, "params.txt has no value for coefficient " + std::to_string(c));
    return x;
}

}  // namespace cg
