// CPU oracle for the design-matrix path -- TEST INFRASTRUCTURE ONLY.
//
// A plain restatement of the reference's algorithm, used by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
// Nothing in the product (the chimes_gb300 library) links or calls this file.
//
// It keeps the reference's loop structure and arithmetic association so that its
// A matrix matches the reference binary on the same inputs:
//   ghosts          FRAME::build_layers            src/ClassDefs.C:2685-2752
//                   BOX::WRAP_ATOM / LAYER_ATOM    src/ClassDefs.C:2064-2164
//   distances       BOX::GET_DISTANCE, get_dist    src/ClassDefs.C:2321-2358, src/functions.h:655-667
//   neighbours      NEIGHBORS::DO_UPDATE_BIG/SMALL src/ClassDefs.C:137-393
//   basis           Cheby::set_polys(+out_of_range) src/Cheby.C:207-443, FCUT::get_fcut src/Fcut.C:17-72
//   2-body rows     Cheby::Deriv_2B                src/Cheby.C:709-883
//   3-body rows     Cheby::Deriv_3B                src/Cheby.C:885-1277
//   4-body rows     Cheby::Deriv_4B                src/Cheby.C:1279-1729
//   charge columns  ZCalc_Ewald_Deriv              src/Ewald.C:477-825 (FITCOUL)
//   row layout, b   A_MAT::PRINT_FRAME             src/A_Matrix.C:210-567
//   MD force        ZCalc                          src/functions.C:815-891
//                   Cheby::Force_all / 3B / 4B     src/Cheby.C:1731-2675
// Parsing and the cluster topology come from the library's host model code
// (model.cpp), whose params.header output is checked byte-for-byte against the
// reference separately.
//
// Build: oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../chimes_lsq-myllfork_gb300/csrc/model.h"

using namespace cg;

namespace {

const double PI_REF = 3.14159265359;   // src/functions.h:48
const double GPA = 6.9476955;          // src/functions.h:45

struct V3 { double x, y, z; };

struct OFrame {
    int natoms, all;
    std::vector<int> type, parent;
    std::vector<V3> coords;   // ALL_COORDS
    Box box;
};

// BOX::GET_DISTANCE (USE_MIC false: ghosts are present)
double get_dist(const Box& b, const V3& a1, const V3& a2, V3& rab) {
    const double* I = b.invr;
    const double* H = b.hmat;
    V3 s1, s2, t;
    s1.x = I[0] * a1.x + I[1] * a1.y + I[2] * a1.z;
    s1.y = I[3] * a1.x + I[4] * a1.y + I[5] * a1.z;
    s1.z = I[6] * a1.x + I[7] * a1.y + I[8] * a1.z;
    s2.x = I[0] * a2.x + I[1] * a2.y + I[2] * a2.z;
    s2.y = I[3] * a2.x + I[4] * a2.y + I[5] * a2.z;
    s2.z = I[6] * a2.x + I[7] * a2.y + I[8] * a2.z;
    t.x = s2.x - s1.x; t.y = s2.y - s1.y; t.z = s2.z - s1.z;
    rab.x = H[0] * t.x + H[1] * t.y + H[2] * t.z;
    rab.y = H[3] * t.x + H[4] * t.y + H[5] * t.z;
    rab.z = H[6] * t.x + H[7] * t.y + H[8] * t.z;
    return std::sqrt(rab.x * rab.x + rab.y * rab.y + rab.z * rab.z);
}

V3 wrap(const Box& b, V3 u) {
    V3 w;
    if (b.is_ortho) {
        int ix = (int)std::floor(u.x / b.lx), iy = (int)std::floor(u.y / b.ly), iz = (int)std::floor(u.z / b.lz);
        w.x = u.x - ix * b.lx; w.y = u.y - iy * b.ly; w.z = u.z - iz * b.lz;
    } else {
        const double* I = b.invr;
        const double* H = b.hmat;
        V3 t;
        t.x = I[0] * u.x + I[1] * u.y + I[2] * u.z;
        t.y = I[3] * u.x + I[4] * u.y + I[5] * u.z;
        t.z = I[6] * u.x + I[7] * u.y + I[8] * u.z;
        int ix = (int)std::floor(t.x), iy = (int)std::floor(t.y), iz = (int)std::floor(t.z);
        t.x -= ix; t.y -= iy; t.z -= iz;
        w.x = H[0] * t.x + H[1] * t.y + H[2] * t.z;
        w.y = H[3] * t.x + H[4] * t.y + H[5] * t.z;
        w.z = H[6] * t.x + H[7] * t.y + H[8] * t.z;
    }
    return w;
}

V3 layer(const Box& b, const V3& r, int n1, int n2, int n3) {
    V3 o;
    if (b.is_ortho) {
        o.x = r.x + n1 * b.ax; o.y = r.y + n2 * b.by; o.z = r.z + n3 * b.cz;
    } else {
        const double* I = b.invr;
        const double* H = b.hmat;
        V3 t;
        t.x = I[0] * r.x + I[1] * r.y + I[2] * r.z;
        t.y = I[3] * r.x + I[4] * r.y + I[5] * r.z;
        t.z = I[6] * r.x + I[7] * r.y + I[8] * r.z;
        t.x += n1; t.y += n2; t.z += n3;
        o.x = H[0] * t.x + H[1] * t.y + H[2] * t.z;
        o.y = H[3] * t.x + H[4] * t.y + H[5] * t.z;
        o.z = H[6] * t.x + H[7] * t.y + H[8] * t.z;
    }
    return o;
}

OFrame make_frame(const Model& m, const Frame& fr) {
    OFrame o;
    o.natoms = fr.natoms;
    o.box = fr.box;
    const int L = m.ctl.nlayers;
    for (int a = 0; a < fr.natoms; ++a) {
        V3 u{fr.xyz[3 * a], fr.xyz[3 * a + 1], fr.xyz[3 * a + 2]};
        o.coords.push_back(wrap(fr.box, u));
        o.type.push_back(fr.type[a]);
        o.parent.push_back(a);
    }
    for (int n1 = -L; n1 <= L; ++n1)
        for (int n2 = -L; n2 <= L; ++n2)
            for (int n3 = -L; n3 <= L; ++n3) {
                if (n1 == 0 && n2 == 0 && n3 == 0) continue;
                for (int a = 0; a < fr.natoms; ++a) {
                    o.coords.push_back(layer(fr.box, o.coords[a], n1, n2, n3));
                    o.type.push_back(fr.type[a]);
                    o.parent.push_back(a);
                }
            }
    o.all = (int)o.coords.size();
    return o;
}

struct Lists {
    std::vector<std::vector<int>> l2, l3, l4, lew;   // lew: LIST_EWALD (FITCOUL)
    double perm[5] = {1, 1, 1, 1, 1};
};

double max_all_cutoffs(const Model& m) {
    double v = -1.0;
    if (m.max_cutoff_2b > v) v = m.max_cutoff_2b;
    if (m.max_cutoff_3b > v) v = m.max_cutoff_3b;
    if (m.max_cutoff_4b > v) v = m.max_cutoff_4b;
    return v;
}

// NEIGHBORS::DO_UPDATE_BIG (pad 0.3) / DO_UPDATE_SMALL
Lists neighbours(const Model& m, const OFrame& fr, bool small, double ewald_cut = 0.0) {
    Lists L;
    L.l2.resize(fr.natoms); L.l3.resize(fr.natoms); L.l4.resize(fr.natoms); L.lew.resize(fr.natoms);
    const double pad = m.ctl.use_neigh ? 0.3 : 1.0e10;
    const double c2 = m.max_cutoff_2b + pad, c3 = m.max_cutoff_3b + pad, c4 = m.max_cutoff_4b + pad;
    const double cew = ewald_cut + pad;
    V3 rab;
    if (small) {
        for (int j = 2; j < 5; ++j) L.perm[j] = L.perm[j - 1] / j;
        for (int a1 = 0; a1 < fr.natoms; ++a1)
            for (int a2 = 0; a2 < fr.all; ++a2) {
                if (a2 == a1) continue;
                double r = get_dist(fr.box, fr.coords[a1], fr.coords[a2], rab);
                if (r < c2) L.l2[a1].push_back(a2);
                if (r < c3) L.l3[a1].push_back(a2);
                if (r < c4) L.l4[a1].push_back(a2);
                if (r < cew) L.lew[a1].push_back(a2);
            }
        return L;
    }
    const int NL = m.ctl.nlayers;
    const Box& b = fr.box;
    double search = m.max_cutoff_2b;
    if (m.max_cutoff_3b > search) search = m.max_cutoff_3b;
    if (m.max_cutoff_4b > search) search = m.max_cutoff_4b;
    if (ewald_cut > search) search = ewald_cut;   // SEARCH_DIST includes EWALD_CUTOFF
    search += pad;
    int nx = (int)std::ceil((2 * NL + 1) * b.extent_x / search) + 2;
    int ny = (int)std::ceil((2 * NL + 1) * b.extent_y / search) + 2;
    int nz = (int)std::ceil((2 * NL + 1) * b.extent_z / search) + 2;
    std::vector<std::vector<int>> bins((size_t)nx * ny * nz);
    auto bin_of = [&](const V3& c, int& ix, int& iy, int& iz) {
        ix = (int)std::floor((c.x - b.xlo + b.extent_x * NL) / search) + 1;
        iy = (int)std::floor((c.y - b.ylo + b.extent_y * NL) / search) + 1;
        iz = (int)std::floor((c.z - b.zlo + b.extent_z * NL) / search) + 1;
    };
    for (int a = 0; a < fr.all; ++a) {
        int ix, iy, iz;
        bin_of(fr.coords[a], ix, iy, iz);
        if (ix < 0 || iy < 0 || iz < 0 || ix >= nx || iy >= ny || iz >= nz)
            throw Error(2, "oracle: out of range binning");
        bins[ix + (size_t)iy * nx + (size_t)iz * nx * ny].push_back(a);
    }
    for (int a1 = 0; a1 < fr.natoms; ++a1) {
        int bx, by, bz;
        bin_of(fr.coords[a1], bx, by, bz);
        for (int i = bx - 1; i <= bx + 1; ++i)
            for (int j = by - 1; j <= by + 1; ++j)
                for (int k = bz - 1; k <= bz + 1; ++k) {
                    const auto& bn = bins[i + (size_t)j * nx + (size_t)k * nx * ny];
                    for (int a2 : bn) {
                        if (a2 == a1) continue;
                        double r = get_dist(b, fr.coords[a1], fr.coords[a2], rab);
                        if (a1 <= fr.parent[a2]) {
                            if (r < c2) L.l2[a1].push_back(a2);
                            if (r < cew) L.lew[a1].push_back(a2);
                            if (r < c3) L.l3[a1].push_back(a2);
                            if (r < c4) L.l4[a1].push_back(a2);
                        }
                    }
                }
    }
    return L;
}

struct Basis {
    const Model& m;
    // Cheby::set_polys / set_polys_out_of_range
    void polys(int pt, double* Tn, double* Tnd, double rlen, double xdiff, double xavg, int snum, double smin) const {
        const PairType& p = m.pairs[pt];
        const double dc = m.deriv_const;
        auto transform = [&](double r, double& x, double& ex) {
            ex = 0.0;
            if (p.trans == TRANS_MORSE) { ex = std::exp(-r / p.lambda); x = (ex - xavg) / xdiff; }
            else if (p.trans == TRANS_INVRSE_R) x = (1.0 / r - xavg) / xdiff;
            else x = (r - xavg) / xdiff;
        };
        auto dxdr = [&](double r, double ex) {
            if (p.trans == TRANS_MORSE) return (-ex / p.lambda) / xdiff;
            if (p.trans == TRANS_INVRSE_R) return -1.0 / (r * r * xdiff);
            return 1.0 / xdiff;
        };
        double x = 0, ex = 0;
        if (rlen >= smin) {
            transform(rlen, x, ex);
            Tn[0] = 1.0; Tn[1] = x; Tnd[0] = 1.0; Tnd[1] = 2.0 * x;
            for (int i = 2; i <= snum; ++i) { Tn[i] = 2.0 * x * Tn[i - 1] - Tn[i - 2]; Tnd[i] = 2.0 * x * Tnd[i - 1] - Tnd[i - 2]; }
            double d = dc * dxdr(rlen, ex);
            for (int i = snum; i >= 1; --i) Tnd[i] = i * d * Tnd[i - 1];
            Tnd[0] = 0.0;
            return;
        }
        transform(smin, x, ex);
        Tn[0] = 1.0; Tn[1] = x;
        if (m.ctl.fix == FIX_ZERO_DERIV) {
            Tnd[0] = 0.0; Tnd[1] = 0.0;
            for (int i = 2; i <= snum; ++i) { Tn[i] = 2.0 * x * Tn[i - 1] - Tn[i - 2]; Tnd[i] = 0.0; }
            return;
        }
        Tnd[0] = 1.0; Tnd[1] = 2.0 * x;
        for (int i = 2; i <= snum; ++i) { Tn[i] = 2.0 * x * Tn[i - 1] - Tn[i - 2]; Tnd[i] = 2.0 * x * Tnd[i - 1] - Tnd[i - 2]; }
        double d = dc * dxdr(smin, ex);
        for (int i = snum; i >= 1; --i) Tnd[i] = i * d * Tnd[i - 1];
        Tnd[0] = 0.0;
        if (m.ctl.fix == FIX_CONSTANT_DERIV) {
            for (int i = 0; i <= snum; ++i) Tn[i] += Tnd[i] * (rlen - smin);
        } else {
            const double dl = m.ctl.smooth;
            double damp = std::exp((rlen - smin) / dl);
            for (int i = 0; i <= snum; ++i) { Tn[i] += dl * (damp - 1.0) * Tnd[i]; Tnd[i] *= damp; }
        }
    }
    void fcut(double& f, double& fd, double r, double rmax) const {
        if (m.ctl.fcut == FCUT_CUBIC) {
            double f0 = 1.0 - r / rmax;
            f = std::pow(f0, 3);
            fd = std::pow(f0, 2);
            fd *= -1.0 * 3 / rmax;
        } else {
            double th = rmax - m.ctl.fcut_offset * rmax;
            if (r < th) { f = 1.0; fd = 0.0; }
            else if (r > rmax) { f = 0.0; fd = 0.0; }
            else {
                double a = (r - th) / (rmax - th) * PI_REF + PI_REF / 2.0;
                double ad = PI_REF / (rmax - th);
                f = 0.5 + 0.5 * std::sin(a);
                fd = 0.5 * std::cos(a) * ad;
            }
        }
    }
};

// Columns of the reference's FORCES / STRESSES arrays: every pair type's 2-body block
// (TOT_SHORT_RANGE); PRINT_FRAME leaves out the HIERARC-excluded ones (skip_2b,
// src/A_Matrix.C:192-208, 240-530) and add_col_of_ones the excluded types' offsets.
int full_2b(const Model& m) { return (int)m.pairs.size() * m.ctl.cheby_order; }
int full_short(const Model& m) { return full_2b(m) + m.num3 + m.num4; }
int printed_col(const Model& m, int c) {   // -1 when skip_2b drops column c
    if (c >= full_2b(m)) return c - full_2b(m) + m.tot_snum;
    const int base = m.pairs[c / m.ctl.cheby_order].col;
    return base < 0 ? -1 : base + c % m.ctl.cheby_order;
}

struct Acc {   // A_MAT::FORCES / STRESSES / FRAME_ENERGIES of one frame
    int C;
    std::vector<double> F;   // [atom][col][3]
    std::vector<double> S;   // [col][6] xx xy xz yy yz zz
    std::vector<double> E;   // [col]
    Acc(int n, int c) : C(c), F((size_t)n * c * 3, 0.0), S((size_t)c * 6, 0.0), E(c, 0.0) {}
    double* f(int a, int col) { return &F[((size_t)a * C + col) * 3]; }
    double* s(int col) { return &S[(size_t)col * 6]; }
};

void stress_add(double* s, double fw, const V3& r, double rl, bool diag, bool all) {
    if (diag) {
        s[0] -= fw * r.x * r.x / rl; s[3] -= fw * r.y * r.y / rl; s[5] -= fw * r.z * r.z / rl;
    } else if (all) {
        s[0] -= fw * r.x * r.x / rl; s[1] -= fw * r.x * r.y / rl; s[2] -= fw * r.x * r.z / rl;
        s[3] -= fw * r.y * r.y / rl; s[4] -= fw * r.y * r.z / rl; s[5] -= fw * r.z * r.z / rl;
    }
}

int pair_index(const Model& m, const OFrame& fr, int a1, int a2) {
    return m.int_pair_map[fr.type[fr.parent[a1]] * m.ctl.natmtyp + fr.type[fr.parent[a2]]];
}

void deriv_2b(const Model& m, const OFrame& fr, const Lists& L, Acc& A, bool fs, bool fsa, bool fe) {
    Basis B{m};
    std::vector<double> Tn(m.ctl.cheby_order + 2), Tnd(m.ctl.cheby_order + 2);
    V3 rab;
    for (int a1 = 0; a1 < fr.natoms; ++a1)
        for (int a2 : L.l2[a1]) {
            int pt = pair_index(m, fr, a1, a2);
            const PairType& p = m.pairs[pt];
            int vstart = pt * p.snum;
            double r = get_dist(fr.box, fr.coords[a1], fr.coords[a2], rab);
            if (!(r > p.smin && r < p.smax)) continue;
            B.polys(pt, Tn.data(), Tnd.data(), r, p.xdiff, p.xavg, p.snum, p.smin);
            double fc, fd;
            B.fcut(fc, fd, r, p.smax);
            int fa2 = fr.parent[a2];
            for (int i = 0; i < p.snum; ++i) {
                double t = L.perm[2] * (fc * Tnd[i + 1] + fd * Tn[i + 1]);
                double* f1 = A.f(a1, vstart + i);
                double* f2 = A.f(fa2, vstart + i);
                double d = t * rab.x / r; f1[0] += d; f2[0] -= d;
                d = t * rab.y / r; f1[1] += d; f2[1] -= d;
                d = t * rab.z / r; f1[2] += d; f2[2] -= d;
                stress_add(A.s(vstart + i), t, rab, r, fs, fsa);
                if (fe) A.E[vstart + i] += L.perm[2] * fc * Tn[i + 1];
            }
        }
}

void deriv_3b(const Model& m, const OFrame& fr, const Lists& L, Acc& A, bool fs, bool fsa, bool fe) {
    Basis B{m};
    const ClusterList& cl = m.trips;
    const int ord = m.ctl.cheby3;
    std::vector<double> T[3], D[3];
    for (int e = 0; e < 3; ++e) { T[e].resize(ord + 2); D[e].resize(ord + 2); }
    const double perm = L.perm[3];
    V3 R[3];
    double rl[3];
    for (int a1 = 0; a1 < fr.natoms; ++a1)
        for (int a2 : L.l3[a1])
            for (int a3 : L.l3[a1]) {
                if (a3 == a2) continue;
                if (perm == 1.0 && fr.parent[a2] > fr.parent[a3]) continue;
                int pts[3] = {pair_index(m, fr, a1, a2), pair_index(m, fr, a1, a3), pair_index(m, fr, a2, a3)};
                int ti[3] = {fr.type[a1], fr.type[a2], fr.type[a3]};
                int id = make_id_int(ti, 3);
                int T3 = cl.int_map[id];
                if (T3 < 0) continue;
                const ClusterType& ct = cl.vec[T3];
                const std::vector<int>& pi = cl.pair_indices[id];
                rl[0] = get_dist(fr.box, fr.coords[a1], fr.coords[a2], R[0]);
                rl[1] = get_dist(fr.box, fr.coords[a1], fr.coords[a3], R[1]);
                rl[2] = get_dist(fr.box, fr.coords[a2], fr.coords[a3], R[2]);
                bool ok = true;
                for (int e = 0; e < 3; ++e) ok = ok && rl[e] < ct.smax[pi[e]];   // FCUT::PROCEED
                if (!ok) continue;
                double fc[3], fd[3];
                for (int e = 0; e < 3; ++e)
                    B.polys(pts[e], T[e].data(), D[e].data(), rl[e], ct.xdiff[pi[e]], ct.xavg[pi[e]], ord, ct.smin[pi[e]]);
                int vstart = full_2b(m);
                for (int t = 0; t < T3; ++t) vstart += cl.vec[t].n_true;
                for (int e = 0; e < 3; ++e) B.fcut(fc[e], fd[e], rl[e], ct.smax[pi[e]]);
                int f2 = fr.parent[a2], f3 = fr.parent[a3];
                for (int p = 0; p < ct.n_allowed; ++p) {
                    int col = vstart + ct.param_indices[p];
                    int pw[3] = {ct.allowed_powers[p][pi[0]], ct.allowed_powers[p][pi[1]], ct.allowed_powers[p][pi[2]]};
                    double d0 = fc[0] * D[0][pw[0]] + fd[0] * T[0][pw[0]];
                    double d1 = fc[1] * D[1][pw[1]] + fd[1] * T[1][pw[1]];
                    double d2 = fc[2] * D[2][pw[2]] + fd[2] * T[2][pw[2]];
                    double w0 = perm * (d0 * fc[1] * fc[2] * T[1][pw[1]] * T[2][pw[2]]);
                    double w1 = perm * (d1 * fc[0] * fc[2] * T[0][pw[0]] * T[2][pw[2]]);
                    double w2 = perm * (d2 * fc[0] * fc[1] * T[0][pw[0]] * T[1][pw[1]]);
                    double* F1 = A.f(a1, col);
                    double* F2 = A.f(f2, col);
                    double* F3 = A.f(f3, col);
                    F1[0] += w0 * R[0].x / rl[0]; F2[0] -= w0 * R[0].x / rl[0];
                    F1[1] += w0 * R[0].y / rl[0]; F2[1] -= w0 * R[0].y / rl[0];
                    F1[2] += w0 * R[0].z / rl[0]; F2[2] -= w0 * R[0].z / rl[0];
                    F1[0] += w1 * R[1].x / rl[1]; F3[0] -= w1 * R[1].x / rl[1];
                    F1[1] += w1 * R[1].y / rl[1]; F3[1] -= w1 * R[1].y / rl[1];
                    F1[2] += w1 * R[1].z / rl[1]; F3[2] -= w1 * R[1].z / rl[1];
                    F2[0] += w2 * R[2].x / rl[2]; F3[0] -= w2 * R[2].x / rl[2];
                    F2[1] += w2 * R[2].y / rl[2]; F3[1] -= w2 * R[2].y / rl[2];
                    F2[2] += w2 * R[2].z / rl[2]; F3[2] -= w2 * R[2].z / rl[2];
                    double* s = A.s(col);
                    stress_add(s, w0, R[0], rl[0], fs, fsa);
                    stress_add(s, w1, R[1], rl[1], fs, fsa);
                    stress_add(s, w2, R[2], rl[2], fs, fsa);
                    if (fe) A.E[col] += fc[0] * fc[1] * fc[2] * T[0][pw[0]] * T[1][pw[1]] * T[2][pw[2]] * perm;
                }
            }
}

void deriv_4b(const Model& m, const OFrame& fr, const Lists& L, Acc& A, bool fs, bool fsa, bool fe) {
    Basis B{m};
    const ClusterList& cl = m.quads;
    const int ord = m.ctl.cheby4;
    std::vector<double> T[6], D[6];
    for (int e = 0; e < 6; ++e) { T[e].resize(ord + 2); D[e].resize(ord + 2); }
    const double perm = L.perm[4];
    V3 R[6];
    double rl[6];
    static const int ea[6] = {0, 0, 0, 1, 1, 2}, eb[6] = {1, 2, 3, 2, 3, 3};
    for (int a1 = 0; a1 < fr.natoms; ++a1)
        for (int a2 : L.l4[a1])
            for (int a3 : L.l4[a1]) {
                if (a3 == a2) continue;
                if (perm == 1.0 && fr.parent[a2] > fr.parent[a3]) continue;
                for (int a4 : L.l4[a1]) {
                    if (a2 == a4 || a3 == a4) continue;
                    if (perm == 1.0 && fr.parent[a3] > fr.parent[a4]) continue;
                    int at[4] = {a1, a2, a3, a4};
                    int pts[6];
                    for (int e = 0; e < 6; ++e) pts[e] = pair_index(m, fr, at[ea[e]], at[eb[e]]);
                    int ti[4] = {fr.type[a1], fr.type[a2], fr.type[a3], fr.type[a4]};
                    int id = make_id_int(ti, 4);
                    int Q = cl.int_map[id];
                    if (Q < 0) continue;
                    for (int e = 0; e < 6; ++e) rl[e] = get_dist(fr.box, fr.coords[at[ea[e]]], fr.coords[at[eb[e]]], R[e]);
                    const ClusterType& ct = cl.vec[Q];
                    const std::vector<int>& pm = cl.pair_indices[id];
                    bool ok = true;
                    for (int e = 0; e < 6 && ok; ++e) ok = rl[e] < ct.smax[pm[e]];
                    if (!ok) continue;
                    for (int e = 0; e < 6; ++e)
                        B.polys(pts[e], T[e].data(), D[e].data(), rl[e], ct.xdiff[pm[e]], ct.xavg[pm[e]], ord, ct.smin[pm[e]]);
                    int vstart = full_2b(m) + m.num3;
                    for (int t = 0; t < Q; ++t) vstart += cl.vec[t].n_true;
                    double fc[6], fd[6];
                    for (int e = 0; e < 6; ++e) B.fcut(fc[e], fd[e], rl[e], ct.smax[pm[e]]);
                    int fid[4] = {a1, fr.parent[a2], fr.parent[a3], fr.parent[a4]};
                    for (int p = 0; p < ct.n_allowed; ++p) {
                        int col = vstart + ct.param_indices[p];
                        int pw[6];
                        for (int e = 0; e < 6; ++e) pw[e] = ct.allowed_powers[p][pm[e]];
                        double dv[6], w[6];
                        for (int e = 0; e < 6; ++e) dv[e] = perm * (fc[e] * D[e][pw[e]] + fd[e] * T[e][pw[e]]);
                        for (int e = 0; e < 6; ++e) {   // force_wo_coeff[e]: deriv * other fcuts * other Tn (src/Cheby.C:1581-1586)
                            double v = dv[e];
                            for (int k = 0; k < 6; ++k) if (k != e) v *= fc[k];
                            for (int k = 0; k < 6; ++k) if (k != e) v *= T[k][pw[k]];
                            w[e] = v;
                        }
                        for (int e = 0; e < 6; ++e) {
                            double* Fa = A.f(fid[ea[e]], col);
                            double* Fb = A.f(fid[eb[e]], col);
                            Fa[0] += w[e] * R[e].x / rl[e]; Fb[0] -= w[e] * R[e].x / rl[e];
                            Fa[1] += w[e] * R[e].y / rl[e]; Fb[1] -= w[e] * R[e].y / rl[e];
                            Fa[2] += w[e] * R[e].z / rl[e]; Fb[2] -= w[e] * R[e].z / rl[e];
                        }
                        double* s = A.s(col);
                        for (int e = 0; e < 6; ++e) stress_add(s, w[e], R[e], rl[e], fs, fsa);
                        double te = fc[0] * fc[1] * fc[2] * fc[3] * fc[4] * fc[5];
                        te *= perm;
                        te *= T[0][pw[0]] * T[1][pw[1]] * T[2][pw[2]] * T[3][pw[3]] * T[4][pw[4]] * T[5][pw[5]];
                        if (fe) A.E[col] += te;
                    }
                }
            }
}

// ZCalc_Ewald_Deriv src/Ewald.C:477-750 (orthorhombic): Q[(p * N + a) * 3 + x], the
// charge-column force of atom a per unit q_i q_j of pair type p.  Real space over
// LIST_EWALD, k space over every atom pair with the per-pair sine tables of
// generate_trig / add_sines (src/Ewald.C:752-825), then the sign flip.
void ewald_add_sines(int kx, int ky, int kz, const std::vector<V3>& S, const std::vector<V3>& C, double& out) {
    V3 sk, ck;
    if (kx >= 0) { sk.x = S[kx].x; ck.x = C[kx].x; } else { sk.x = -S[-kx].x; ck.x = C[-kx].x; }
    if (ky >= 0) { sk.y = S[ky].y; ck.y = C[ky].y; } else { sk.y = -S[-ky].y; ck.y = C[-ky].y; }
    if (kz >= 0) { sk.z = S[kz].z; ck.z = C[kz].z; } else { sk.z = -S[-kz].z; ck.z = C[-kz].z; }
    const double syz = sk.y * ck.z + ck.y * sk.z;
    const double cyz = ck.y * ck.z - sk.y * sk.z;
    out = sk.x * cyz + ck.x * syz;
}

void ewald_deriv(const Model& m, const OFrame& fr, const Frame& raw, const Lists& L, const EwaldParams& ep,
                 std::vector<double>& Q) {
    const int N = fr.natoms, np = (int)m.pairs.size();
    Q.assign((size_t)np * N * 3, 0.0);
    auto q = [&](int p, int a) { return &Q[((size_t)p * N + a) * 3]; };
    const double PI = 3.14159265359, ke = 1.0;
    const double alpha = ep.alpha, alphasq = alpha * alpha, r_cut = ep.rc;
    const int kmax = ep.kmax, ksqmax = 50;
    const Box& b = fr.box;
    const double Volume = b.vol;
    std::vector<int> kv;   // kx, ky, kz triples
    std::vector<double> kfac;
    for (int kx = 0; kx <= kmax; kx++)
        for (int ky = 0; ky <= kmax; ky++)
            for (int kz = 0; kz <= kmax; kz++) {
                const int ksq = kx * kx + ky * ky + kz * kz;
                if (ksq != 0 && ksq < ksqmax) {
                    const double rx = (2.0 * PI / b.ax) * kx, ry = (2.0 * PI / b.by) * ky, rz = (2.0 * PI / b.cz) * kz;
                    const double rksq = rx * rx + ry * ry + rz * rz;
                    kv.push_back(kx); kv.push_back(ky); kv.push_back(kz);
                    kfac.push_back(std::exp(-rksq / (4.0 * alphasq)) / rksq);
                }
            }
    const double perm_scale = L.perm[2];
    V3 R;
    for (int a1 = 0; a1 < N; a1++)
        for (int a2 : L.lew[a1]) {
            const int fidx = fr.parent[a2];
            const int p = pair_index(m, fr, a1, a2);
            const double rl = get_dist(b, fr.coords[a1], fr.coords[a2], R);
            if (rl < r_cut) {
                double t = ((-2.0 / std::sqrt(PI)) * std::exp(-1 * alpha * alpha * rl * rl) * rl * alpha -
                            std::erfc(alpha * rl)) / (rl * rl);
                t *= -1.0; t *= 2.0; t *= ke; t *= 0.5 / rl; t *= perm_scale;
                double* qa = q(p, a1);
                double* qb = q(p, fidx);
                qa[0] += t * R.x; qa[1] += t * R.y; qa[2] += t * R.z;
                qb[0] -= t * R.x; qb[1] -= t * R.y; qb[2] -= t * R.z;
            }
        }
    std::vector<V3> S(kmax + 1), C(kmax + 1);
    const int totk = (int)kfac.size();
    for (int a1 = 0; a1 < N; a1++)
        for (int a2 = 0; a2 < a1; a2++) {
            const int p = pair_index(m, fr, a1, a2);
            V3 rv{raw.xyz[3 * a2] - raw.xyz[3 * a1], raw.xyz[3 * a2 + 1] - raw.xyz[3 * a1 + 1],
                  raw.xyz[3 * a2 + 2] - raw.xyz[3 * a1 + 2]};
            S[0] = {0.0, 0.0, 0.0};
            C[0] = {1.0, 1.0, 1.0};
            if (kmax >= 1) {
                S[1] = {std::sin(2.0 * M_PI * rv.x / b.ax), std::sin(2.0 * M_PI * rv.y / b.by),
                        std::sin(2.0 * M_PI * rv.z / b.cz)};
                C[1] = {std::cos(2.0 * M_PI * rv.x / b.ax), std::cos(2.0 * M_PI * rv.y / b.by),
                        std::cos(2.0 * M_PI * rv.z / b.cz)};
            }
            for (int ik = 2; ik <= kmax; ik++) {
                S[ik].x = S[ik - 1].x * C[1].x + C[ik - 1].x * S[1].x;
                S[ik].y = S[ik - 1].y * C[1].y + C[ik - 1].y * S[1].y;
                S[ik].z = S[ik - 1].z * C[1].z + C[ik - 1].z * S[1].z;
                C[ik].x = C[ik - 1].x * C[1].x - S[ik - 1].x * S[1].x;
                C[ik].y = C[ik - 1].y * C[1].y - S[ik - 1].y * S[1].y;
                C[ik].z = C[ik - 1].z * C[1].z - S[ik - 1].z * S[1].z;
            }
            double* qa = q(p, a1);
            double* qb = q(p, a2);
            for (int ik = 0; ik < totk; ik++) {
                const int kx = kv[3 * ik], ky = kv[3 * ik + 1], kz = kv[3 * ik + 2];
                const double rkx = (2.0 * PI / b.ax) * kx, rky = (2.0 * PI / b.by) * ky, rkz = (2.0 * PI / b.cz) * kz;
                const double Kfac = kfac[ik];
                double t1, t2 = 0.0, t3 = 0.0, t4 = 0.0;
                ewald_add_sines(kx, ky, kz, S, C, t1);
                t1 *= ke; t1 *= 2.0; t1 *= Kfac * 0.5 * (4 * PI / Volume);
                if (ky > 0) {
                    ewald_add_sines(kx, -ky, kz, S, C, t2);
                    t2 *= ke; t2 *= 2.0; t2 *= Kfac * 0.5 * (4 * PI / Volume);
                    if (kz > 0) {
                        ewald_add_sines(kx, -ky, -kz, S, C, t3);
                        t3 *= ke; t3 *= 2.0; t3 *= Kfac * 0.5 * (4 * PI / Volume);
                    }
                }
                if (kz > 0) {
                    ewald_add_sines(kx, ky, -kz, S, C, t4);
                    t4 *= ke; t4 *= 2.0; t4 *= Kfac * 0.5 * (4 * PI / Volume);
                }
                if (kx > 0) { t1 *= 2.0; t2 *= 2.0; t3 *= 2.0; t4 *= 2.0; }
                qa[0] += (t1 + t2 + t3 + t4) * rkx;
                qa[1] += (t1 - t2 - t3 + t4) * rky;
                qa[2] += (t1 + t2 - t3 - t4) * rkz;
                qb[0] -= (t1 + t2 + t3 + t4) * rkx;
                qb[1] -= (t1 - t2 - t3 + t4) * rky;
                qb[2] -= (t1 + t2 - t3 - t4) * rkz;
            }
        }
    for (double& v : Q) v *= -1.0;
}

// One frame's A rows (dense, lda >= tot_all) and b values.
void frame_rows_out(const Model& m, const Frame& fr, int fi, bool small, double* out, int64_t lda, double* b) {
    OFrame of = make_frame(m, fr);
    EwaldParams ep;
    if (m.ncoul > 0) {
        if (!fr.box.is_ortho) throw Error(2, "oracle: Ewald needs an orthorhombic cell");
        ep = ewald_params(fr.natoms, fr.box);
    }
    Lists L = neighbours(m, of, small, m.ncoul > 0 ? ep.rc : 0.0);
    RowLayout rl = frame_rows(m, fi, fr.natoms);
    const bool fs = rl.stress_rows == 3, fsa = rl.stress_rows == 9, fe = rl.energy_rows > 0;
    const int CF = full_short(m);
    Acc A(fr.natoms, CF);
    if (m.ctl.cheby_order > 0) deriv_2b(m, of, L, A, fs, fsa, fe);
    if (m.ctl.use3) deriv_3b(m, of, L, A, fs, fsa, fe);
    if (m.ctl.use4) deriv_4b(m, of, L, A, fs, fsa, fe);
    const double iv = 1.0 / fr.box.vol;
    if (fs || fsa)
        for (int c = 0; c < CF; ++c)
            for (int k = 0; k < 6; ++k) A.S[(size_t)c * 6 + k] *= iv;
    int64_t row = 0;
    auto put = [&](int64_t r, int c, double v) { out[r * lda + c] = v; };
    auto put_short = [&](int64_t r, int c, double v) {   // full column c -> printed column
        const int pc = printed_col(m, c);
        if (pc >= 0) out[r * lda + pc] = v;
    };
    std::vector<int> count(m.ctl.natmtyp, 0);
    for (int a = 0; a < fr.natoms; ++a) count[fr.type[a]]++;
    const int nener = m.ctl.fit_ener ? m.ctl.natmtyp : 0;   // types scanned; excluded ones print nothing
    auto ecol = [&](int t) { return m.ener_col[t]; };
    std::vector<double> Q;
    if (m.ncoul > 0) ewald_deriv(m, of, fr, L, ep, Q);
    for (int a = 0; a < fr.natoms; ++a)
        for (int x = 0; x < 3; ++x, ++row) {
            for (int c = 0; c < CF; ++c) put_short(row, c, A.f(a, c)[x]);
            for (int p = 0; p < m.ncoul; ++p) put(row, m.tot_short + p, Q[((size_t)p * fr.natoms + a) * 3 + x]);
            for (int t = 0; t < nener; ++t) if (ecol(t) >= 0) put(row, m.tot_short + m.ncoul + ecol(t), 0.0);
            b[row] = fr.force[3 * a + x];
        }
    if (rl.stress_rows) {
        const int* idx;
        static const int d3[3] = {0, 3, 5}, a9[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
        idx = fs ? d3 : a9;
        const double xx = fr.stress_diag[0], yy = fr.stress_diag[1], zz = fr.stress_diag[2];
        const double xy = fr.stress_off[0], xz = fr.stress_off[1], yz = fr.stress_off[2];
        const double bd3[3] = {xx, yy, zz}, b9[9] = {xx, xy, xz, xy, yy, yz, xz, yz, zz};
        for (int k = 0; k < rl.stress_rows; ++k, ++row) {
            for (int c = 0; c < CF; ++c) put_short(row, c, A.S[(size_t)c * 6 + idx[k]]);
            for (int t = 0; t < nener; ++t) if (ecol(t) >= 0) put(row, m.tot_short + ecol(t), 0.0);
            b[row] = (fs ? bd3[k] : b9[k]) / GPA;
        }
    }
    for (int k = 0; k < rl.energy_rows; ++k, ++row) {
        for (int c = 0; c < CF; ++c) put_short(row, c, A.E[c]);
        for (int t = 0; t < nener; ++t) if (ecol(t) >= 0) put(row, m.tot_short + ecol(t), (double)count[t]);
        b[row] = fr.energy;
    }
}

// ---------------------------------------------------------------- MD force
// ZCalc with Cheby::Force_all / Force_3B / Force_4B: the same lists and basis as
// the fit, contracted with the coefficients x (one per A column).  F gets
// SYSTEM.ACCEL (forces, kcal/mol/A); S gets [TOT_POT_ENER, PRESSURE_XYZ/(3V),
// PRESSURE_TENSORS_XYZ_ALL/V (3x3 row-major)].
struct MdOut {
    std::vector<V3> F;
    double E = 0, P = 0, W[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
};

void md_tensor(MdOut& o, double fw, const V3& R) {   // fw already divided by r
    o.W[0][0] -= fw * R.x * R.x; o.W[0][1] -= fw * R.x * R.y; o.W[0][2] -= fw * R.x * R.z;
    o.W[1][1] -= fw * R.y * R.y; o.W[1][2] -= fw * R.y * R.z;
    o.W[2][2] -= fw * R.z * R.z;
    o.W[1][0] = o.W[0][1]; o.W[2][0] = o.W[0][2]; o.W[2][1] = o.W[1][2];
}

void md_force_2b(const Model& m, const OFrame& fr, const Lists& L, const double* x, double pd, double ps, MdOut& o) {
    Basis B{m};
    std::vector<double> Tn(m.ctl.cheby_order + 2), Tnd(m.ctl.cheby_order + 2);
    V3 rab;
    const double perm = L.perm[2];
    for (int a1 = 0; a1 < fr.natoms; ++a1)
        for (int a2 : L.l2[a1]) {
            int pt = pair_index(m, fr, a1, a2);
            const PairType& p = m.pairs[pt];
            double r = get_dist(fr.box, fr.coords[a1], fr.coords[a2], rab);
            if (!(r < p.smax)) continue;   // r < s_min included (src/Cheby.C:1834)
            B.polys(pt, Tn.data(), Tnd.data(), r, p.xdiff, p.xavg, p.snum, p.smin);
            double fc, fd;
            B.fcut(fc, fd, r, p.smax);
            int fa2 = fr.parent[a2];
            for (int i = 0; i < p.snum; ++i) {
                double coeff = p.col < 0 ? 0.0 : perm * x[p.col + i];   // HIERARC-excluded pairs: 0
                o.E += coeff * fc * Tn[i + 1];
                double deriv = fc * Tnd[i + 1] + fd * Tn[i + 1];
                o.P -= coeff * deriv * r;
                md_tensor(o, coeff * deriv / r, rab);
                o.F[a1].x += coeff * deriv * rab.x / r; o.F[a1].y += coeff * deriv * rab.y / r;
                o.F[a1].z += coeff * deriv * rab.z / r;
                o.F[fa2].x -= coeff * deriv * rab.x / r; o.F[fa2].y -= coeff * deriv * rab.y / r;
                o.F[fa2].z -= coeff * deriv * rab.z / r;
            }
            double rpen = (r - pd < p.smin) ? p.smin + pd - r : 0.0;   // src/Cheby.C:1900-1968
            if (rpen > 0.0) {
                double coeff = -3.0 * rpen * rpen * ps;
                o.F[a1].x += coeff * rab.x / r; o.F[a1].y += coeff * rab.y / r; o.F[a1].z += coeff * rab.z / r;
                o.F[fa2].x -= coeff * rab.x / r; o.F[fa2].y -= coeff * rab.y / r; o.F[fa2].z -= coeff * rab.z / r;
                o.E += rpen * rpen * rpen * ps;
                o.P -= coeff * r;
                md_tensor(o, coeff / r, rab);
            }
        }
}

// Force_3B (src/Cheby.C:2024-2300) over the fit's triplet enumeration.
void md_force_3b(const Model& m, const OFrame& fr, const Lists& L, const double* x, MdOut& o) {
    Basis B{m};
    const ClusterList& cl = m.trips;
    const int ord = m.ctl.cheby3;
    std::vector<double> T[3], D[3];
    for (int e = 0; e < 3; ++e) { T[e].resize(ord + 2); D[e].resize(ord + 2); }
    const double perm = L.perm[3];
    V3 R[3];
    double rl[3];
    for (int a1 = 0; a1 < fr.natoms; ++a1)
        for (int a2 : L.l3[a1])
            for (int a3 : L.l3[a1]) {
                if (a3 == a2) continue;
                if (perm == 1.0 && fr.parent[a2] > fr.parent[a3]) continue;
                int pts[3] = {pair_index(m, fr, a1, a2), pair_index(m, fr, a1, a3), pair_index(m, fr, a2, a3)};
                int ti[3] = {fr.type[a1], fr.type[a2], fr.type[a3]};
                int id = make_id_int(ti, 3);
                int T3 = cl.int_map[id];
                if (T3 < 0) continue;
                const ClusterType& ct = cl.vec[T3];
                const std::vector<int>& pi = cl.pair_indices[id];
                rl[0] = get_dist(fr.box, fr.coords[a1], fr.coords[a2], R[0]);
                rl[1] = get_dist(fr.box, fr.coords[a1], fr.coords[a3], R[1]);
                rl[2] = get_dist(fr.box, fr.coords[a2], fr.coords[a3], R[2]);
                bool ok = true;
                for (int e = 0; e < 3; ++e) ok = ok && rl[e] < ct.smax[pi[e]];
                if (!ok) continue;
                double fc[3], fd[3];
                for (int e = 0; e < 3; ++e)
                    B.polys(pts[e], T[e].data(), D[e].data(), rl[e], ct.xdiff[pi[e]], ct.xavg[pi[e]], ord, ct.smin[pi[e]]);
                for (int e = 0; e < 3; ++e) B.fcut(fc[e], fd[e], rl[e], ct.smax[pi[e]]);
                int vstart = m.tot_snum;
                for (int t = 0; t < T3; ++t) vstart += cl.vec[t].n_true;
                int fid[3] = {a1, fr.parent[a2], fr.parent[a3]};
                static const int ea[3] = {0, 0, 1}, eb[3] = {1, 2, 2};
                for (int p = 0; p < ct.n_allowed; ++p) {
                    double coeff = perm * x[vstart + ct.param_indices[p]];
                    int pw[3] = {ct.allowed_powers[p][pi[0]], ct.allowed_powers[p][pi[1]], ct.allowed_powers[p][pi[2]]};
                    o.E += coeff * fc[0] * fc[1] * fc[2] * T[0][pw[0]] * T[1][pw[1]] * T[2][pw[2]];
                    double d[3], f[3];
                    for (int e = 0; e < 3; ++e) d[e] = fc[e] * D[e][pw[e]] + fd[e] * T[e][pw[e]];
                    f[0] = coeff * d[0] * fc[1] * fc[2] * T[1][pw[1]] * T[2][pw[2]];
                    f[1] = coeff * d[1] * fc[0] * fc[2] * T[0][pw[0]] * T[2][pw[2]];
                    f[2] = coeff * d[2] * fc[0] * fc[1] * T[0][pw[0]] * T[1][pw[1]];
                    for (int e = 0; e < 3; ++e) {
                        o.P -= f[e] * rl[e];
                        double fw = f[e] / rl[e];
                        md_tensor(o, fw, R[e]);
                        V3& A = o.F[fid[ea[e]]];
                        V3& Bv = o.F[fid[eb[e]]];
                        A.x += fw * R[e].x; A.y += fw * R[e].y; A.z += fw * R[e].z;
                        Bv.x -= fw * R[e].x; Bv.y -= fw * R[e].y; Bv.z -= fw * R[e].z;
                    }
                }
            }
}

// Force_4B (src/Cheby.C:2303-2675) over the fit's quadruplet enumeration.
void md_force_4b(const Model& m, const OFrame& fr, const Lists& L, const double* x, MdOut& o) {
    Basis B{m};
    const ClusterList& cl = m.quads;
    const int ord = m.ctl.cheby4;
    std::vector<double> T[6], D[6];
    for (int e = 0; e < 6; ++e) { T[e].resize(ord + 2); D[e].resize(ord + 2); }
    const double perm = L.perm[4];
    V3 R[6];
    double rl[6];
    static const int ea[6] = {0, 0, 0, 1, 1, 2}, eb[6] = {1, 2, 3, 2, 3, 3};
    for (int a1 = 0; a1 < fr.natoms; ++a1)
        for (int a2 : L.l4[a1])
            for (int a3 : L.l4[a1]) {
                if (a3 == a2) continue;
                if (perm == 1.0 && fr.parent[a2] > fr.parent[a3]) continue;
                for (int a4 : L.l4[a1]) {
                    if (a2 == a4 || a3 == a4) continue;
                    if (perm == 1.0 && fr.parent[a3] > fr.parent[a4]) continue;
                    int at[4] = {a1, a2, a3, a4};
                    int pts[6];
                    for (int e = 0; e < 6; ++e) pts[e] = pair_index(m, fr, at[ea[e]], at[eb[e]]);
                    int ti[4] = {fr.type[a1], fr.type[a2], fr.type[a3], fr.type[a4]};
                    int id = make_id_int(ti, 4);
                    int Q = cl.int_map[id];
                    if (Q < 0) continue;
                    for (int e = 0; e < 6; ++e) rl[e] = get_dist(fr.box, fr.coords[at[ea[e]]], fr.coords[at[eb[e]]], R[e]);
                    const ClusterType& ct = cl.vec[Q];
                    const std::vector<int>& pm = cl.pair_indices[id];
                    bool ok = true;
                    for (int e = 0; e < 6 && ok; ++e) ok = rl[e] < ct.smax[pm[e]];
                    if (!ok) continue;
                    for (int e = 0; e < 6; ++e)
                        B.polys(pts[e], T[e].data(), D[e].data(), rl[e], ct.xdiff[pm[e]], ct.xavg[pm[e]], ord, ct.smin[pm[e]]);
                    double fc[6], fd[6];
                    for (int e = 0; e < 6; ++e) B.fcut(fc[e], fd[e], rl[e], ct.smax[pm[e]]);
                    int vstart = m.tot_snum + m.num3;
                    for (int t = 0; t < Q; ++t) vstart += cl.vec[t].n_true;
                    int fid[4] = {a1, fr.parent[a2], fr.parent[a3], fr.parent[a4]};
                    for (int p = 0; p < ct.n_allowed; ++p) {
                        double coeff = perm * x[vstart + ct.param_indices[p]];
                        int pw[6];
                        for (int e = 0; e < 6; ++e) pw[e] = ct.allowed_powers[p][pm[e]];
                        double te = coeff;
                        for (int e = 0; e < 6; ++e) te *= fc[e];
                        for (int e = 0; e < 6; ++e) te *= T[e][pw[e]];
                        o.E += te;
                        for (int e = 0; e < 6; ++e) {
                            double f = coeff * (fc[e] * D[e][pw[e]] + fd[e] * T[e][pw[e]]);
                            for (int k = 0; k < 6; ++k) if (k != e) f *= fc[k];
                            for (int k = 0; k < 6; ++k) if (k != e) f *= T[k][pw[k]];
                            o.P -= f * rl[e];
                            double fw = f / rl[e];
                            md_tensor(o, fw, R[e]);
                            V3& A = o.F[fid[ea[e]]];
                            V3& Bv = o.F[fid[eb[e]]];
                            A.x += fw * R[e].x; A.y += fw * R[e].y; A.z += fw * R[e].z;
                            Bv.x -= fw * R[e].x; Bv.y -= fw * R[e].y; Bv.z -= fw * R[e].z;
                        }
                    }
                }
            }
}

void md_force_frame(const Model& m, const Frame& fr, bool small, const double* x, bool offsets, double pd, double ps,
                    double* F, double* S) {
    OFrame of = make_frame(m, fr);
    Lists L = neighbours(m, of, small);
    MdOut o;
    o.F.assign(fr.natoms, V3{0, 0, 0});
    if (offsets)
        for (int a = 0; a < fr.natoms; ++a)
            if (m.ener_col[fr.type[a]] >= 0) o.E += x[m.tot_short + m.ncoul + m.ener_col[fr.type[a]]];
    if (m.ctl.cheby_order > 0) md_force_2b(m, of, L, x, pd, ps, o);
    if (m.ctl.use3) md_force_3b(m, of, L, x, o);
    if (m.ctl.use4) md_force_4b(m, of, L, x, o);
    for (int a = 0; a < fr.natoms; ++a) { F[3 * a] = o.F[a].x; F[3 * a + 1] = o.F[a].y; F[3 * a + 2] = o.F[a].z; }
    const double V = fr.box.vol;
    S[0] = o.E;
    S[1] = o.P / (3.0 * V);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) S[2 + 3 * i + j] = o.W[i][j] / V;
}

std::vector<Frame> frames_from_arrays(const Model& m, int nframes, const int* natoms, const int* types,
                                      const double* xyz, const double* cell) {
    std::vector<Frame> frames(nframes);
    int64_t a0 = 0;
    for (int f = 0; f < nframes; ++f) {
        Frame& fr = frames[f];
        fr.natoms = natoms[f];
        fr.type.assign(types + a0, types + a0 + fr.natoms);
        fr.xyz.assign(xyz + 3 * a0, xyz + 3 * (a0 + fr.natoms));
        fr.force.assign(3 * (size_t)fr.natoms, 0.0);
        const double* c = cell + 9 * (size_t)f;
        Box& b = fr.box;
        b.ax = c[0]; b.ay = c[1]; b.az = c[2]; b.bx = c[3]; b.by = c[4]; b.bz = c[5];
        b.cx = c[6]; b.cy = c[7]; b.cz = c[8];
        b.update_cell();
        a0 += fr.natoms;
    }
    return frames;
}

thread_local std::string g_err;

}  // namespace

// Frame number in the trajectory (NSTRESS / NENER): the reader's index, which SKPFRMS
// keeps for the frames it selects (src/chimes_lsq.C:305-322 passes i on).
static int traj_index(const std::vector<Frame>& fr, int k) { return fr[k].index >= 0 ? fr[k].index : k; }

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

// Columns and rows of an input (for sizing the output buffers).
int oracle_sizes(const char* fm_setup, const char* xyzf, int nframes, int64_t* nrows, int* ncols) {
    try {
        Model m = load_model(fm_setup);
        Box box;
        std::vector<Frame> fr = xyzf ? read_xyzf(m, xyzf, nframes > 0 ? nframes : m.ctl.nframes, 0, box)
                                     : read_frames(m);
        if (nframes > 0 && (size_t)nframes < fr.size()) fr.resize(nframes);   // the first nframes frames
        int64_t r = 0;
        for (size_t f = 0; f < fr.size(); ++f) r += frame_rows(m, traj_index(fr, (int)f), fr[f].natoms).total();
        *nrows = r;
        *ncols = m.tot_all;
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 2;
    }
}

// Assemble A (row-major, lda) and b for frames [first, first+count) of the trajectory,
// with nthreads OpenMP threads over frames (the reference's MPI frame split).
int oracle_assemble(const char* fm_setup, const char* xyzf, int nframes, int first, int count, int nthreads,
                    double* A, int64_t lda, double* b) {
    try {
        Model m = load_model(fm_setup);
        Box box;
        std::vector<Frame> fr = xyzf ? read_xyzf(m, xyzf, nframes > 0 ? nframes : m.ctl.nframes, 0, box)
                                     : read_frames(m);
        if (nframes > 0 && (size_t)nframes < fr.size()) fr.resize(nframes);   // the first nframes frames
        if (count <= 0) count = (int)fr.size() - first;
        std::vector<int64_t> ofs(count + 1, 0);
        std::vector<char> small(count, 0);
        bool sm = false;
        for (int k = 0; k < first + count; ++k) {
            sm = frame_is_small(m, fr[k].box, sm);
            if (k >= first) small[k - first] = sm;
        }
        for (int k = 0; k < count; ++k)
            ofs[k + 1] = ofs[k] + frame_rows(m, traj_index(fr, first + k), fr[first + k].natoms).total();
        std::string err;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
        for (int k = 0; k < count; ++k) {
            try {
                frame_rows_out(m, fr[first + k], traj_index(fr, first + k), small[k], A + ofs[k] * lda, lda, b + ofs[k]);
            } catch (const std::exception& e) {
#pragma omp critical
                err = e.what();
            }
        }
        if (!err.empty()) throw Error(2, err);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 2;
    }
}

// MD force of independent configurations (each decides the small-cell convention
// alone): forces [3 * sum natoms] and 11 scalars per frame (see md_force_frame).
int oracle_md_force(const char* fm_setup, int nframes, const int* natoms, const int* types, const double* xyz,
                    const double* cell, const double* x, int nx, int offsets, double pen_dist, double pen_scale,
                    int nthreads, double* F, double* S) {
    try {
        Model m = load_model(fm_setup);
        if (nx != m.tot_all) throw Error(1, "coefficient count does not match the model");
        std::vector<Frame> fr = frames_from_arrays(m, nframes, natoms, types, xyz, cell);
        std::vector<int64_t> ofs(nframes + 1, 0);
        for (int f = 0; f < nframes; ++f) ofs[f + 1] = ofs[f] + natoms[f];
        std::string err;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
        for (int f = 0; f < nframes; ++f) {
            try {
                bool small = frame_is_small(m, fr[f].box, false);
                md_force_frame(m, fr[f], small, x, offsets != 0, pen_dist, pen_scale, F + 3 * ofs[f], S + 11 * f);
            } catch (const std::exception& e) {
#pragma omp critical
                err = e.what();
            }
        }
        if (!err.empty()) throw Error(2, err);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return 2;
    }
}

}  // extern "C"
