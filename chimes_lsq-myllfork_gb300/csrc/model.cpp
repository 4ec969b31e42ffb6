// Host-side model: fm_setup.in parser, pair / cluster topology, .xyzf reader.
// See model.h for the reference functions each part follows.
//
// Built with -ffp-contract=off: the box set-up arithmetic must round exactly like
// the reference's (its pair and cluster sets are decided by FP64 comparisons).
#include "model.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <sstream>

namespace cg {

static const int MAX_ATOM_TYPES = 10;   // src/functions.h:34
static const double FORCE_CONV = 627.50960803 * 1.889725989;   // src/ClassDefs.C:2632-2634

// ------------------------------------------------------------------ helpers

static void strip_comments(std::string& line) {   // src/util.C:54-67
    size_t pos = line.find('!');
    if (pos != std::string::npos) line.erase(pos);
    pos = line.find("##");
    if (pos != std::string::npos) line.erase(pos);
}

static int parse_space(std::string line, std::vector<std::string>& tokens) {   // src/util.C:26-50
    strip_comments(line);
    std::stringstream ss(line);
    tokens.clear();
    std::string buf;
    while (ss >> buf) tokens.push_back(buf);
    return (int)tokens.size();
}

[[noreturn]] static void fail(const std::string& msg) { throw Error(2, msg); }

static bool to_bool(const std::string& s) {
    if (s == "true" || s == "True" || s == "TRUE" || s == "T" || s == "t") return true;
    if (s == "false" || s == "False" || s == "FALSE" || s == "F" || s == "f") return false;
    fail("expected a boolean, got: " + s);
}
static int to_int(const std::string& s) {
    try { size_t n; int v = std::stoi(s, &n); return v; } catch (...) { fail("expected an integer, got: " + s); }
}
static double to_double(const std::string& s) {
    try { return std::stod(s); } catch (...) { fail("expected a number, got: " + s); }
}

struct Listing {
    std::vector<std::vector<std::string>> lines;
    const std::string& at(size_t i, size_t j) const {
        if (i >= lines.size()) fail("input was not found for line " + std::to_string(i));
        if (j >= lines[i].size()) fail("not enough tokens in input line " + std::to_string(i));
        return lines[i][j];
    }
    size_t size(size_t i) const {
        if (i >= lines.size()) fail("input was not found for line " + std::to_string(i));
        return lines[i].size();
    }
    bool keyword(size_t i, const char* kw) const {   // "# KEYWORD #"
        const auto& l = lines[i];
        return l.size() >= 3 && l[0] == "#" && l[2] == "#" && l[1] == kw;
    }
    std::string joined(size_t i) const {
        std::string s;
        for (size_t k = 0; k < lines[i].size(); ++k) { if (k) s += ' '; s += lines[i][k]; }
        return s;
    }
};

static Listing read_listing(const std::string& path) {   // INPUT::READ_FILE src/input.C:109-162
    std::ifstream in(path);
    if (!in.is_open()) fail("cannot open input file: " + path);
    Listing L;
    std::string line;
    int kick = 0;
    bool ended = false;
    while (std::getline(in, line)) {
        strip_comments(line);
        std::vector<std::string> toks;
        if (parse_space(line, toks) == 0) continue;
        L.lines.push_back(toks);
        if (line.find("# ENDFILE #") != std::string::npos) { ended = true; break; }
        if (++kick == 1000) break;
    }
    if (!ended) fail("did not find \"# ENDFILE #\" in " + path);
    return L;
}

int make_id_int(const int* types, int n) {
    int sum = 0, weight = 1;
    for (int i = 0; i < n; ++i) { sum += weight * (types[i] + 1); weight *= MAX_ATOM_TYPES; }
    return sum;
}

// Cheby::set_cheby_params src/Cheby.C:102-139
static void set_cheby_params(double smin, double smax, double lambda, int trans, double& xmin,
                             double& xmax, double& xdiff, double& xavg) {
    switch (trans) {
        case TRANS_MORSE: xmin = std::exp(-smax / lambda); xmax = std::exp(-smin / lambda); break;
        case TRANS_INVRSE_R: xmin = 1.0 / smax; xmax = 1.0 / smin; break;
        default: xmin = smin; xmax = smax; break;
    }
    xavg = 0.5 * (xmin + xmax);
    xdiff = 0.5 * (xmax - xmin);
}

static int trans_from_string(const std::string& s) {   // Cheby::get_trans_type src/Cheby.C:167-184
    if (s == "MORSE") return TRANS_MORSE;
    if (s == "INVRSE_R") return TRANS_INVRSE_R;
    if (s == "DEFAULT" || s == "NONE") return TRANS_NONE;
    fail("bad Chebyshev transformation type: " + s);
}
static const char* trans_string(int t) {
    return t == TRANS_MORSE ? "MORSE" : (t == TRANS_INVRSE_R ? "INVRSE_R" : "NONE");
}

// ------------------------------------------------------------ control parse

static void parse_controls(const Listing& L, Controls& c, const std::string& dir) {
    const size_t N = L.lines.size();
    for (size_t i = 0; i < N; ++i) {   // TRJFILE  src/input.C:290-430
        if (L.size(i) > 1 && L.at(i, 1) == "TRJFILE") {
            if (L.size(i + 1) == 1) {
                c.infile.push_back(L.at(i + 1, 0));
                c.force_flags.push_back(""); c.stress_flags.push_back(""); c.energy_flags.push_back("");
            } else if (L.size(i + 1) == 2) {
                // "MULTI <list>": <nfiles>, then per file <nframes> <file> [T] [F S E flags]
                std::string lp = L.at(i + 1, 1);
                if (!lp.empty() && lp[0] != '/') lp = dir + "/" + lp;
                std::ifstream multi(lp);
                if (!multi.is_open()) fail("Cannot open MULTI file: " + L.at(i + 1, 1));
                std::string line;
                std::vector<std::string> t;
                std::getline(multi, line);
                if (parse_space(line, t) != 1) fail("Expected to read <nfiles>, got: " + line);
                const int nfiles = to_int(t[0]);
                for (int j = 0; j < nfiles; ++j) {
                    std::getline(multi, line);
                    const int n = parse_space(line, t);
                    if (n != 2 && n != 3 && n != 5 && n != 6)
                        fail("Expected <nframes> <filename> [temperature] [F_flag S_flag E_flag], got: " + line);
                    c.infile_frames.push_back(to_int(t[0]));
                    c.infile.push_back(t[1]);
                    if (n >= 5) {
                        c.force_flags.push_back(t[n - 3] != "None" ? t[n - 3] : "");
                        c.stress_flags.push_back(t[n - 2] != "None" ? t[n - 2] : "");
                        c.energy_flags.push_back(t[n - 1] != "None" ? t[n - 1] : "");
                    } else {
                        c.force_flags.push_back(""); c.stress_flags.push_back(""); c.energy_flags.push_back("");
                    }
                }
                for (int k = (int)c.infile_frames.size() - 1; k >= 0; --k)   // files with no frames are dropped
                    if (c.infile_frames[k] < 1) {
                        c.infile.erase(c.infile.begin() + k);
                        c.infile_frames.erase(c.infile_frames.begin() + k);
                        c.force_flags.erase(c.force_flags.begin() + k);
                        c.stress_flags.erase(c.stress_flags.begin() + k);
                        c.energy_flags.erase(c.energy_flags.begin() + k);
                    }
            } else {
                fail("TRJFILE expects one file name or MULTI <list>");
            }
            break;
        }
    }
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "WRAPTRJ")) { if (i + 1 < N && L.size(i + 1) == 1) { c.wrap = to_bool(L.at(i + 1, 0)); break; } }
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "SPLITFI")) { c.split_files = to_bool(L.at(i + 1, 0)); break; }
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "HIERARC")) { c.hierarchical = to_bool(L.at(i + 1, 0)); break; }
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "NFRAMES")) { c.nframes = to_int(L.at(i + 1, 0)); break; }
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "NLAYERS")) { c.nlayers = to_int(L.at(i + 1, 0)); break; }
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "FITCOUL")) { c.fit_coul = to_bool(L.at(i + 1, 0)); break; }
    for (size_t i = 0; i < N; ++i) {   // FITSTRS src/input.C:536-577
        if (L.keyword(i, "FITSTRS")) {
            const std::string& v = L.at(i + 1, 0);
            if (v == "first" || v == "First" || v == "FIRST") { c.fit_stress = true; c.nstress = to_int(L.at(i + 1, 1)); }
            else if (v == "all" || v == "All" || v == "ALL" || v == "A" || v == "a") c.fit_stress_all = true;
            else if (v == "firstall" || v == "FirstAll" || v == "FIRSTALL") { c.fit_stress_all = true; c.nstress = to_int(L.at(i + 1, 1)); }
            else c.fit_stress = to_bool(v);
            break;
        }
    }
    for (size_t i = 0; i < N; ++i) {   // FITENER src/input.C:578-604 (no break: last one wins)
        if (L.keyword(i, "FITENER")) {
            const std::string& v = L.at(i + 1, 0);
            if (v == "first" || v == "First" || v == "FIRST") { c.fit_ener = true; c.nener = to_int(L.at(i + 1, 1)); }
            else c.fit_ener = to_bool(v);
        }
    }
    for (size_t i = 0; i < N; ++i) {   // PAIRTYP src/input.C:606-689
        if (L.keyword(i, "PAIRTYP")) {
            c.ff_type = L.at(i + 1, 0);
            if (c.ff_type != "CHEBYSHEV") fail("unrecognized pair type: " + c.ff_type);
            c.cheby_order = to_int(L.at(i + 1, 1));
            c.cheby3 = L.size(i + 1) >= 3 ? to_int(L.at(i + 1, 2)) : 0;
            c.use3 = c.cheby3 > 0;
            c.cheby4 = L.size(i + 1) >= 4 ? to_int(L.at(i + 1, 3)) : 0;
            c.use4 = c.cheby4 > 0;
            c.range_low = L.size(i + 1) > 4 ? (double)to_int(L.at(i + 1, 4)) : -1.0;
            c.range_high = L.size(i + 1) > 5 ? (double)to_int(L.at(i + 1, 5)) : 1.0;
            if (c.range_low < -1 || c.range_low > 1 || c.range_high < -1 || c.range_high > 1 ||
                c.range_high < c.range_low)
                fail("bad Chebyshev transformation range in PAIRTYP");
            break;
        }
    }
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "CHBTYPE")) c.trans = trans_from_string(L.at(i + 1, 0));
    for (size_t i = 0; i < N; ++i) {   // CHEBYFIX src/input.C:713-747
        if (L.keyword(i, "CHEBYFIX")) {
            const std::string& v = L.at(i + 1, 0);
            if (v == "ZERO_DERIV") c.fix = FIX_ZERO_DERIV;
            else if (v == "CONSTANT_DERIV") c.fix = FIX_CONSTANT_DERIV;
            else if (v == "SMOOTH") { c.fix = FIX_SMOOTH; c.smooth = to_double(L.at(i + 1, 1)); }
            else fail("CHEBYFIX was not recognized");
        }
    }
    for (size_t i = 0; i < N; ++i) {   // USENEIG src/input.C:1694-1720
        if (L.keyword(i, "USENEIG")) {
            c.use_neigh = to_bool(L.at(i + 1, 0));
            if (L.size(i + 1) == 2 && c.use_neigh) {
                if (L.at(i + 1, 1) == "SMALL") c.force_small = true;
                else fail("unrecognized USENEIG option: " + L.at(i + 1, 1));
            }
            break;
        }
    }
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "SKPFRMS")) { c.skip_frames = to_int(L.at(i + 1, 0)); break; }
}

// ------------------------------------------------------------ cluster topology

static void cluster_init(ClusterType& ct, int natoms, int npairs) {
    ct.natoms = natoms; ct.npairs = npairs;
    ct.atom_names.assign(natoms, ""); ct.atom_indices.assign(natoms, 0); ct.pair_names.assign(npairs, "");
    ct.smax.assign(npairs, 0); ct.smin.assign(npairs, 0); ct.xmin.assign(npairs, 0);
    ct.xmax.assign(npairs, 0); ct.xavg.assign(npairs, 0); ct.xdiff.assign(npairs, 0);
}

// CLUSTER::permute_atom_indices src/Cluster.C:255-366
static void permute_atom_indices(ClusterType& ct, int idx, const std::vector<int>& unsorted,
                                 std::vector<int> perm, int unique_index, int equiv_index) {
    const int n = ct.natoms;
    if (idx < n) {
        int count = 1;
        for (int i = idx; i < n - 1; ++i) {
            if (ct.atom_names[i + 1] == ct.atom_names[i]) ++count; else break;
        }
        do {
            permute_atom_indices(ct, idx + count, unsorted, perm, unique_index, equiv_index);
        } while (std::next_permutation(perm.begin() + idx, perm.begin() + idx + count));
        return;
    }
    std::vector<std::vector<int>> pm(n, std::vector<int>(n, 0));
    int c = 0;
    for (int i = 0; i < n; ++i) for (int j = i + 1; j < n; ++j) pm[i][j] = unsorted[c++];
    for (int k = 0; k < n; ++k) for (int l = 0; l < k; ++l) pm[k][l] = pm[l][k];
    std::vector<int> pp(ct.npairs);
    c = 0;
    for (int i = 0; i < n; ++i) for (int j = i + 1; j < n; ++j) pp[c++] = pm[perm[i]][perm[j]];
    auto it = ct.allowed_map.find(pp);
    if (it == ct.allowed_map.end()) {
        ct.allowed_powers.push_back(pp);
        ct.power_count.push_back(1);
        ct.allowed_map.emplace(pp, (int)ct.allowed_powers.size() - 1);
        ct.param_indices.push_back(unique_index);
        ct.equiv_indices.push_back(equiv_index);
    } else {
        ++ct.power_count[it->second];
    }
}

static void store_permutations(ClusterType& ct, const std::vector<int>& unsorted) {   // :181-246
    if (ct.allowed_map.count(unsorted)) return;
    ct.unique_powers.push_back(unsorted);
    std::vector<int> perm(ct.natoms);
    for (int i = 0; i < ct.natoms; ++i) perm[i] = i;
    int equiv_index = (int)ct.allowed_powers.size();
    permute_atom_indices(ct, 0, unsorted, perm, (int)ct.unique_powers.size() - 1, equiv_index);
}

static void build_loop(ClusterType& ct, int indx, int order, std::vector<int> powers) {   // :115-158
    if (indx < ct.npairs) {
        for (int p = 0; p < order; ++p) { powers[indx] = p; build_loop(ct, indx + 1, order, powers); }
        return;
    }
    std::vector<bool> rep(ct.natoms, false);
    int c = 0;
    for (int i = 0; i < ct.natoms; ++i)
        for (int j = i + 1; j < ct.natoms; ++j)
            if (powers[c++] > 0) { rep[i] = true; rep[j] = true; }
    for (int i = 0; i < ct.natoms; ++i) if (!rep[i]) return;
    store_permutations(ct, powers);
}

static void cluster_build(ClusterType& ct, int order) {   // CLUSTER::build :27-113
    if (!ct.excluded) build_loop(ct, 0, order, std::vector<int>(ct.npairs, 0));
    ct.n_true = (int)ct.unique_powers.size();
    ct.n_allowed = (int)ct.param_indices.size();
    for (int j = 0, k = 0; j < (int)ct.allowed_powers.size();) {
        for (; k < (int)ct.allowed_powers.size() && ct.param_indices[j] == ct.param_indices[k]; ++k)
            if (ct.power_count[k] != ct.power_count[j]) fail("assumption of equal power counts was incorrect");
        j = k;
    }
}

// CLUSTER::map_indices_int src/Cluster.C:1768-1878
static void map_indices_int(const ClusterType& ct, const std::vector<int>& atom_type_idx,
                            std::vector<int>& pair_map) {
    const int n = ct.natoms;
    std::vector<std::vector<int>> pidx(n, std::vector<int>(n, -1));
    int c = 0;
    for (int j = 0; j < n; ++j) for (int k = j + 1; k < n; ++k) { pidx[j][k] = c; pidx[k][j] = c; ++c; }
    std::vector<bool> used(n, false);
    std::vector<int> rev(n, -1);
    for (int m = 0; m < n; ++m)
        for (int q = 0; q < n; ++q)
            if (atom_type_idx[m] == ct.atom_indices[q] && !used[q]) { rev[m] = q; used[q] = true; break; }
    for (int j = 0; j < n; ++j) if (rev[j] < 0) fail("bad reverse index while mapping cluster pairs");
    int m = 0;
    pair_map.assign(ct.npairs, -1);
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) pair_map[m++] = pidx[rev[i]][rev[j]];
}

static bool is_excluded(const ClusterList& cl, std::vector<std::string> names) {   // :1486-1505
    std::sort(names.begin(), names.end());
    for (const auto& ex : cl.exclude) {
        int k = 0;
        for (; k < cl.natoms; ++k) if (ex[k] != names[k]) break;
        if (k == cl.natoms) return true;
    }
    return false;
}

static void build_pairs_loop(Model& m, ClusterList& cl, int index, std::vector<int> ai,
                             const std::vector<std::string>& chems, int& count) {   // :1293-1484
    const int nt = (int)chems.size();
    const int n = cl.natoms, np = cl.npairs;
    if (index < n) {
        for (int i = 0; i < nt; ++i) { ai[index] = i; build_pairs_loop(m, cl, index + 1, ai, chems, count); }
        return;
    }
    std::vector<std::string> names(n), pn(np), pnu(np);
    for (int i = 0; i < n; ++i) names[i] = chems[ai[i]];
    std::sort(names.begin(), names.end());
    int c2 = 0;
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            pn[c2] = m.pairs[m.pair_map[names[i] + names[j]]].prpr;
            pnu[c2] = m.pairs[m.pair_map[chems[ai[i]] + chems[ai[j]]]].prpr;
            ++c2;
        }
    bool new_pair = true;
    int map_index = -1;
    for (int i = 0; i < count; ++i) {
        int k = 0;
        for (; k < np; ++k) if (cl.vec[i].pair_names[k] != pn[k]) break;
        if (k == np) { new_pair = false; map_index = i; break; }
    }
    bool excl = is_excluded(cl, names);
    if (new_pair) {
        if (count >= (int)cl.vec.size()) { cl.vec.emplace_back(); cluster_init(cl.vec.back(), n, np); }
        ClusterType& ct = cl.vec[count];
        c2 = 0;
        for (int i = 0; i < n; ++i) {
            ct.atom_names[i] = names[i];
            size_t j = 0;
            for (; j < m.atom_types.size(); ++j) if (names[i] == m.atom_types[j]) break;
            if (j == m.atom_types.size()) fail("could not find an element type for " + names[i]);
            ct.atom_indices[i] = m.atom_type_idx[j];
            for (int k = i + 1; k < n; ++k) { ct.pair_names[c2] = pn[c2]; ++c2; }
        }
        if (!excl) map_index = count; else ct.excluded = true;
        ct.index = count;
        ++count;
    }
    std::string all;
    for (const auto& s : pnu) all += s;
    if (excl) map_index = -1;
    cl.map.emplace(all, map_index);
    cl.map_reverse.emplace(map_index, all);
    int id = make_id_int(ai.data(), n);
    cl.int_map[id] = map_index;
    cl.pair_indices[id].assign(np, -1);
    if (map_index >= 0) {
        map_indices_int(cl.vec[map_index], ai, cl.pair_indices[id]);
        cl.int_map_reverse[map_index] = id;
    }
}

static void process_cutoff_params(Model& m, ClusterList& cl, bool is_max) {   // :771-954
    std::vector<std::string>& input = is_max ? cl.smax_input : cl.smin_input;
    const int np = cl.npairs;
    if (!input.empty()) {
        std::vector<std::string> t;
        if (parse_space(input[0], t) < 5) fail("not enough tokens: " + input[0]);
        if (t[3] == "ALL") {
            double v = to_double(t[4]);
            for (auto& ct : cl.vec) {
                for (int j = 0; j < np; ++j) (is_max ? ct.smax : ct.smin)[j] = v;
                (is_max ? ct.special_smax : ct.special_smin) = true;
            }
        } else if (t[3] == "SPECIFIC") {
            int nspec = to_int(t[4]);
            for (int s = 0; s < nspec; ++s) {
                if (s + 1 >= (int)input.size()) fail("missing SPECIFIC cutoff line");
                std::vector<std::string> tk;
                if (parse_space(input[s + 1], tk) != 2 * np + 1) fail("wrong number of arguments: " + input[s + 1]);
                auto it = cl.map.find(tk[0]);
                if (it == cl.map.end()) fail("did not find a map for cluster named " + tk[0]);
                int ci = it->second;
                if (ci < 0) continue;
                for (int i = 0; i < np; ++i) {
                    std::string pname = m.pairs[m.pair_map[tk[i + 1]]].prpr;
                    double v = to_double(tk[i + np + 1]);
                    for (int j = 0; j < np; ++j) {
                        if (pname == cl.vec[ci].pair_names[j]) (is_max ? cl.vec[ci].smax : cl.vec[ci].smin)[j] = v;
                        (is_max ? cl.vec[ci].special_smax : cl.vec[ci].special_smin) = true;
                    }
                }
            }
        }
    }
    if (is_max) {
        double v = -1.0;
        for (auto& ct : cl.vec) for (int j = 0; j < np; ++j) if (ct.smax[j] > v) v = ct.smax[j];
        cl.max_cutoff = v;
    }
}

static void default_cutoffs(const Model& m, ClusterList& cl) {   // set_default_smaxim/sminim :606-655
    for (auto& ct : cl.vec) {
        for (int i = 0; i < cl.npairs; ++i) {
            size_t j = 0;
            for (; j < m.pairs.size(); ++j) if (m.pairs[j].prpr == ct.pair_names[i]) break;
            if (j == m.pairs.size()) fail("a default cutoff could not be set for " + ct.pair_names[i]);
            if (!ct.special_smax) ct.smax[i] = m.pairs[j].smax;
            if (!ct.special_smin) ct.smin[i] = m.pairs[j].smin;
        }
    }
}

static int factorial(int n) { int r = 1; for (int i = 2; i <= n; ++i) r *= i; return r; }

static void build_cluster_list(Model& m, ClusterList& cl, int natoms, int order) {
    cl.natoms = natoms;
    cl.npairs = natoms * (natoms - 1) / 2;
    int nt = m.ctl.natmtyp;
    cl.nclusters = factorial(nt + natoms - 1) / factorial(natoms) / factorial(nt - 1);
    cl.vec.assign(cl.nclusters, ClusterType());
    for (auto& ct : cl.vec) cluster_init(ct, natoms, cl.npairs);
    if (order <= 0) { cl.vec.clear(); cl.nclusters = 0; return; }
    // build_pairs src/Cluster.C:1245-1290
    std::vector<std::string> chems;
    for (const auto& p : m.pairs) {
        if (std::find(chems.begin(), chems.end(), p.atm1) == chems.end()) chems.push_back(p.atm1);
    }
    int dim = 1;
    for (int i = 0; i < natoms; ++i) dim *= MAX_ATOM_TYPES;
    cl.int_map.assign(dim, -1);
    cl.int_map_reverse.assign(cl.nclusters, -1);
    cl.pair_indices.assign(dim, std::vector<int>(cl.npairs, -1));
    int count = 0;
    build_pairs_loop(m, cl, 0, std::vector<int>(natoms, 0), chems, count);
    cl.nclusters = (int)cl.vec.size();
    for (auto& ct : cl.vec) cluster_build(ct, order);
    default_cutoffs(m, cl);
    process_cutoff_params(m, cl, true);
    process_cutoff_params(m, cl, false);
    // CLUSTER::set_cheby_vals src/Cluster.C:1746-1765
    for (auto& ct : cl.vec) {
        for (int i = 0; i < cl.npairs; ++i) {
            size_t j = 0;
            for (; j < m.pairs.size(); ++j) if (ct.pair_names[i] == m.pairs[j].prpr) break;
            if (j == m.pairs.size()) fail("set_cheby_vals: no match for atom pair " + ct.pair_names[i]);
            set_cheby_params(ct.smin[i], ct.smax[i], m.pairs[j].lambda, m.pairs[0].trans, ct.xmin[i],
                             ct.xmax[i], ct.xdiff[i], ct.xavg[i]);
        }
    }
}

// ------------------------------------------------------------ topology parse

static void parse_topology(const Listing& L, Model& m) {
    const size_t N = L.lines.size();
    Controls& c = m.ctl;
    for (size_t i = 0; i < N; ++i)
        if (L.keyword(i, "NATMTYP")) { c.natmtyp = to_int(L.at(i + 1, 0)); }
    if (c.natmtyp <= 0 || c.natmtyp > MAX_ATOM_TYPES) fail("NATMTYP must be between 1 and 10");
    int npair = c.natmtyp * (c.natmtyp + 1) / 2;
    m.pairs.assign(npair, PairType());
    for (auto& p : m.pairs) { p.range_low = c.range_low; p.range_high = c.range_high; }
    // TYPEIDX src/input.C:916-1042
    double sumchg = 0;
    bool found_typeidx = false;
    for (size_t i = 0; i < N && !found_typeidx; ++i) {
        if (!L.keyword(i, "TYPEIDX")) continue;
        found_typeidx = true;
        m.atom_type_idx.assign(c.natmtyp, 0);
        m.atom_types.assign(c.natmtyp, "");
        for (int j = 0; j < c.natmtyp; ++j) {
            PairType& p = m.pairs[j];
            p.pairidx = j;
            p.trans = c.trans;
            m.atom_type_idx[j] = to_int(L.at(i + 1 + j, 0)) - 1;
            if (m.atom_type_idx[j] < 0 || m.atom_type_idx[j] >= c.natmtyp) fail("bad atom index in TYPEIDX section");
            p.t1 = m.atom_type_idx[j];
            p.atm1 = L.at(i + 1 + j, 1);
            m.atom_types[j] = p.atm1;
            if (!c.fit_coul) p.chg1 = to_double(L.at(i + 1 + j, 2));
            else { p.chrgsgn = L.at(i + 1 + j, 2); p.chg1 = 0.0; }
            sumchg += std::fabs(p.chg1);
            p.mass1 = to_double(L.at(i + 1 + j, 3));
            p.atm2 = p.atm1; p.t2 = p.t1; p.chg2 = p.chg1; p.mass2 = p.mass1;
            p.prpr = p.atm1 + p.atm2;
        }
    }
    if (!found_typeidx) fail("missing # TYPEIDX # section");
    if (!c.fit_coul && sumchg > 0) c.use_partial_charges = true;
    int t = c.natmtyp;
    for (int i = 0; i < c.natmtyp; ++i)
        for (int j = i + 1; j < c.natmtyp; ++j) {
            PairType& p = m.pairs[t];
            p.pairidx = t; p.trans = m.pairs[i].trans;
            p.atm1 = m.pairs[i].atm1; p.t1 = m.pairs[i].t1;
            p.atm2 = m.pairs[j].atm1; p.t2 = m.pairs[j].t1;
            p.chg1 = m.pairs[i].chg1; p.chg2 = m.pairs[j].chg1;
            p.mass1 = m.pairs[i].mass1; p.mass2 = m.pairs[j].mass1;
            p.prpr = p.atm1 + p.atm2;
            ++t;
        }
    for (int i = 0; i < c.natmtyp; ++i)
        for (int j = 0; j < c.natmtyp; ++j)
            for (int k = 0; k < npair; ++k) {
                const PairType& pk = m.pairs[k];
                if ((m.pairs[i].atm1 == pk.atm1 && m.pairs[j].atm1 == pk.atm2) ||
                    (m.pairs[j].atm1 == pk.atm1 && m.pairs[i].atm1 == pk.atm2))
                    m.pair_map.emplace(m.pairs[i].atm1 + m.pairs[j].atm2, k);
            }
    // CHARGE CONSTRAINTS  INPUT::PARSE_TOPOLOGY_CHGCONS src/input.C:1148-1200: npair-1 lines of
    // npair pair names, npair values and the force (last token)
    if (c.fit_coul) {
        for (size_t i = 0; i < N; ++i) {
            if (L.size(i) < 2 || L.at(i, 0) + " " + L.at(i, 1) != "CHARGE CONSTRAINTS:") continue;
            for (int n = 0; n < npair - 1; ++n) {
                const size_t li = i + 1 + n;
                ChargeConstraint cc;
                for (int j = 0; j < npair; ++j) {
                    auto it = m.pair_map.find(L.at(li, j));
                    if (it == m.pair_map.end()) fail("unknown pair in CHARGE CONSTRAINTS: " + L.at(li, j));
                    cc.pair.push_back(it->second);
                }
                for (int j = 0; j < npair; ++j) cc.value.push_back(to_double(L.at(li, npair + j)));
                cc.force = to_double(L.at(li, L.size(li) - 1));
                m.charge_constraints.push_back(cc);
            }
            break;
        }
    }
    // EXCLUDE nB INTERACTION  src/input.C:753-874, CLUSTER_LIST::read_exclude src/Cluster.C:1508-1526
    auto read_exclude = [&](const char* tag, std::vector<std::vector<std::string>>& ex, int natoms) {
        for (size_t i = 0; i < N; ++i) {
            if (L.size(i) < 4) continue;
            if (L.at(i, 0) + " " + L.at(i, 1) + " " + L.at(i, 2) != tag) continue;
            int nex = to_int(L.at(i, 3));
            for (int k = 1; k <= nex; ++k) {
                if ((int)L.size(i + k) != natoms) fail("wrong number of atoms in exclude command");
                std::vector<std::string> v = L.lines[i + k];
                std::sort(v.begin(), v.end());
                ex.push_back(v);
            }
            break;
        }
    };
    // HIERARC: EXCLUDE 1B / 2B INTERACTION lists (INPUT::PARSE_TOPOLOGY_EXCLUDE
    // src/input.C:753-842): atom type names, and pair names matched in either order
    if (c.hierarchical) {
        for (size_t i = 0; i < N; ++i) {
            if (L.size(i) < 4 || L.at(i, 0) + " " + L.at(i, 1) + " " + L.at(i, 2) != "EXCLUDE 1B INTERACTION:") continue;
            const int nex = to_int(L.at(i, 3));
            for (int j = 1; j <= nex; ++j)
                for (int k = 0; k < c.natmtyp; ++k)
                    if (L.at(i + j, 0) == m.atom_types[k]) m.excl1b.push_back(m.atom_type_idx[k]);
            break;
        }
        for (size_t i = 0; i < N; ++i) {
            if (L.size(i) < 4 || L.at(i, 0) + " " + L.at(i, 1) + " " + L.at(i, 2) != "EXCLUDE 2B INTERACTION:") continue;
            const int nex = to_int(L.at(i, 3));
            for (int j = 1; j <= nex; ++j)
                for (size_t k = 0; k < m.pairs.size(); ++k) {
                    const PairType& p = m.pairs[k];
                    if ((p.atm1 == L.at(i + j, 0) && p.atm2 == L.at(i + j, 1)) ||
                        (p.atm1 == L.at(i + j, 1) && p.atm2 == L.at(i + j, 0)))
                        m.excl2b.push_back((int)k);
                }
            break;
        }
    }
    read_exclude("EXCLUDE 3B INTERACTION:", m.trips.exclude, 3);
    read_exclude("EXCLUDE 4B INTERACTION:", m.quads.exclude, 4);
    // PAIRIDX src/input.C:1044-1102
    for (size_t ci = 0; ci < N; ++ci) {
        if (!L.keyword(ci, "PAIRIDX")) continue;
        for (int i = 0; i < npair; ++i) {
            std::string key = L.at(ci + 1 + i, 1) + L.at(ci + 1 + i, 2);
            auto it = m.pair_map.find(key);
            if (it == m.pair_map.end()) fail("unknown pair in PAIRIDX: " + key);
            PairType& p = m.pairs[it->second];
            p.pairidx = it->second;
            p.smin = to_double(L.at(ci + 1 + i, 3));
            p.smax = to_double(L.at(ci + 1 + i, 4));
            p.lambda = to_double(L.at(ci + 1 + i, 6));
            if (p.smax > m.max_cutoff_2b) {
                m.max_cutoff_2b = p.smax; m.max_cutoff_3b = p.smax; m.max_cutoff_4b = p.smax;
            }
        }
        break;
    }
    // build_int_pair_map src/functions.C:1055-1095
    m.int_pair_map.assign(c.natmtyp * c.natmtyp, -1);
    for (int i = 0; i < c.natmtyp; ++i)
        for (int j = 0; j < c.natmtyp; ++j)
            m.int_pair_map[m.atom_type_idx[i] * c.natmtyp + m.atom_type_idx[j]] =
                m.pair_map[m.atom_types[i] + m.atom_types[j]];
    for (auto& p : m.pairs) set_cheby_params(p.smin, p.smax, p.lambda, p.trans, p.xmin, p.xmax, p.xdiff, p.xavg);
    // SPECIAL nB S_MINIM / S_MAXIM  src/input.C:1207-1282, read_cutoff_params src/Cluster.C:1018-1043
    auto read_special = [&](const char* tag, std::vector<std::string>& out) {
        for (size_t i = 0; i < N; ++i) {
            if (L.size(i) < 4) continue;
            if (L.at(i, 0) + " " + L.at(i, 1) + " " + L.at(i, 2) != tag) continue;
            out.push_back(L.joined(i));
            if (L.size(i) < 5) fail("not enough tokens: " + L.joined(i));
            if (L.at(i, 3) == "SPECIFIC") {
                int ns = to_int(L.at(i, 4));
                for (int k = 1; k <= ns; ++k) out.push_back(L.joined(i + k));
            }
            break;
        }
    };
    read_special("SPECIAL 3B S_MINIM:", m.trips.smin_input);
    read_special("SPECIAL 4B S_MINIM:", m.quads.smin_input);
    read_special("SPECIAL 3B S_MAXIM:", m.trips.smax_input);
    read_special("SPECIAL 4B S_MAXIM:", m.quads.smax_input);
    // FCUTTYP src/input.C:1283-1301, FCUT::parse_input src/Fcut.C:143-159
    for (size_t i = 0; i < N; ++i) {
        if (!L.keyword(i, "FCUTTYP")) continue;
        c.fcut_line = L.joined(i + 1);
        break;
    }
    {
        std::vector<std::string> tk;
        parse_space(c.fcut_line, tk);
        if (tk.empty()) fail("empty FCUTTYP");
        if (tk[0] == "CUBIC") c.fcut = FCUT_CUBIC;
        else if (tk[0] == "TERSOFF") {
            c.fcut = FCUT_TERSOFF;
            if (tk.size() < 2) fail("TERSOFF cutoff needs an offset");
            c.fcut_offset = to_double(tk[1]);
        } else fail("unknown cutoff type " + tk[0]);
    }
}

Model load_model(const std::string& path) {
    Model m;
    size_t slash = path.find_last_of('/');
    m.dir = slash == std::string::npos ? std::string(".") : path.substr(0, slash);
    Listing L = read_listing(path);
    parse_controls(L, m.ctl, m.dir);
    parse_topology(L, m);
    Controls& c = m.ctl;
    // RUN_SANITY_LSQ src/input.C:1306-1338
    if (c.wrap && c.nlayers > 0) c.wrap = false;
    if (c.fit_coul && (c.fit_stress || c.fit_stress_all || c.fit_ener))
        fail("FITCOUL with stress or energy rows: the reference prints no charge columns on those rows");
    if (c.use_partial_charges && (c.fit_stress || c.fit_stress_all || c.fit_ener))
        fail("fixed charges with stress or energy rows: only the force labels are corrected (SubtractEwaldForces)");
    if (c.nlayers < 1) fail("NLAYERS must be >= 1 (ghost-atom images); NLAYERS 0 is not supported by this library");
    // main: src/chimes_lsq.C:198-248
    // 2-body blocks in pair order without the HIERARC-excluded ones (A_MAT::skip_2b
    // src/A_Matrix.C:192-208 drops them when PRINT_FRAME writes a row)
    m.tot_snum = 0;
    for (size_t k = 0; k < m.pairs.size(); ++k) {
        PairType& p = m.pairs[k];
        p.snum = c.cheby_order; p.snum3 = c.cheby3; p.snum4 = c.cheby4; p.trans = c.trans;
        const bool ex = std::find(m.excl2b.begin(), m.excl2b.end(), (int)k) != m.excl2b.end();
        p.col = ex ? -1 : m.tot_snum;
        if (!ex) m.tot_snum += p.snum;
    }
    for (auto& p : m.pairs) set_cheby_params(p.smin, p.smax, p.lambda, p.trans, p.xmin, p.xmax, p.xdiff, p.xavg);
    m.deriv_const = (m.pairs[0].range_high - m.pairs[0].range_low) / 2.0;
    build_cluster_list(m, m.trips, 3, c.use3 ? c.cheby3 : 0);
    build_cluster_list(m, m.quads, 4, c.use4 ? c.cheby4 : 0);
    if (c.use3) m.max_cutoff_3b = m.trips.max_cutoff;
    if (c.use4) m.max_cutoff_4b = m.quads.max_cutoff;
    m.num3 = 0; m.num4 = 0;
    if (c.use3) for (auto& ct : m.trips.vec) m.num3 += ct.n_true;
    if (c.use4) for (auto& ct : m.quads.vec) m.num4 += ct.n_true;
    m.tot_short = m.tot_snum + m.num3 + m.num4;
    m.ncoul = c.fit_coul ? (int)m.pairs.size() : 0;
    if (m.ncoul > 0 && !m.excl2b.empty()) fail("HIERARC 2-body exclusion with FITCOUL: the solver script refuses it");
    // energy-offset columns: one per atom type not excluded (A_MAT::add_col_of_ones
    // src/A_Matrix.C:155-175)
    int nen = 0;
    m.ener_col.assign(c.natmtyp, -1);
    for (int t = 0; t < c.natmtyp; ++t)
        if (std::find(m.excl1b.begin(), m.excl1b.end(), t) == m.excl1b.end()) m.ener_col[t] = nen++;
    m.tot_all = m.tot_short + m.ncoul + (c.fit_ener ? nen : 0);
    // JOB_CONTROL::LSQ_SETUP src/ClassDefs.C:2761-2785
    if ((c.fit_stress || c.fit_stress_all) && c.nstress == -1) c.nstress = c.nframes;
    if (c.fit_ener && c.nener == -1) c.nener = c.nframes;
    if (c.infile.size() == 1 && c.infile_frames.empty()) c.infile_frames.push_back(c.nframes);
    return m;
}

// ------------------------------------------------------------ header writers

static void cluster_print_special(std::ostream& h, const ClusterType& ct, const std::string& mr, bool smin) {
    if (ct.excluded) return;   // CLUSTER::print_special src/Cluster.C:423-460
    if (smin) {
        if (ct.special_smin) h << " " << mr << " ";
        for (int i = 0; i < ct.npairs; ++i) h << ct.pair_names[i] << " ";
        h << std::fixed << std::setprecision(5);
        for (int i = 0; i < ct.npairs; ++i) h << ct.smin[i] << " ";
    } else {
        if (ct.special_smax) h << mr << " ";
        for (int i = 0; i < ct.npairs; ++i) h << ct.pair_names[i] << " ";
        h << std::fixed << std::setprecision(5);
        for (int i = 0; i < ct.npairs; ++i) h << ct.smax[i] << " ";
    }
    h << std::endl;
}

static void list_print_special(std::ostream& h, const ClusterList& cl) {   // src/Cluster.C:1670-1710
    if (cl.nclusters == 0 || cl.vec.empty()) return;
    int found = 0;
    for (auto& ct : cl.vec) if (ct.special_smin && !ct.excluded) ++found;
    auto mr = [&](int i) { auto it = cl.map_reverse.find(i); return it == cl.map_reverse.end() ? std::string() : it->second; };
    if (found > 0) {
        h << std::endl << "SPECIAL " << cl.natoms << "B S_MINIM: SPECIFIC " << found << std::endl;
        for (size_t i = 0; i < cl.vec.size(); ++i) if (cl.vec[i].special_smin) cluster_print_special(h, cl.vec[i], mr((int)i), true);
    }
    found = 0;
    for (auto& ct : cl.vec) if (ct.special_smax && !ct.excluded) ++found;
    if (found > 0) {
        h << std::endl << "SPECIAL " << cl.natoms << "B S_MAXIM: SPECIFIC " << found << std::endl;
        for (size_t i = 0; i < cl.vec.size(); ++i) if (cl.vec[i].special_smax) cluster_print_special(h, cl.vec[i], mr((int)i), false);
    }
}

static void list_print_header(std::ostream& h, const ClusterList& cl, int natoms, int order) {
    h << std::endl << "ATOM PAIR " << (natoms == 3 ? "TRIPLETS" : "QUADRUPLETS") << ": ";
    if (order == 0 || cl.nclusters == 0) { h << 0 << std::endl; return; }
    h << cl.vec.size() << std::endl << std::endl;
    for (const auto& ct : cl.vec) {   // CLUSTER::print_header src/Cluster.C:463-508
        h << " INDEX: " << ct.index << " ATOMS: ";
        for (int q = 0; q < ct.natoms; ++q) { h << ct.atom_names[q]; if (q < ct.npairs - 1) h << " "; }
        h << std::endl << " PAIRS: ";
        for (int q = 0; q < ct.npairs; ++q) { h << ct.pair_names[q]; if (q < ct.npairs - 1) h << " "; }
        if (ct.excluded) h << " EXCLUDED:\n";
        else {
            h << "  " << ct.n_true << " parameters, " << ct.n_allowed << " total parameters " << std::endl;
            h << "     index  |  powers  |  equiv index  |  param index  " << std::endl;
            h << "   ----------------------------------------------------" << std::endl;
            for (size_t j = 0; j < ct.allowed_powers.size(); ++j) {
                h << "      " << std::setw(6) << std::fixed << std::left << j << " ";
                h << " ";
                for (int q = 0; q < ct.npairs; ++q) h << std::setw(2) << std::fixed << std::left << ct.allowed_powers[j][q] << " ";
                h << "       " << std::setw(8) << ct.equiv_indices[j] << " ";
                h << "       " << std::setw(8) << ct.param_indices[j] << std::endl;
            }
        }
        h << std::endl;
    }
}

std::string params_header_text(const Model& m) {   // print_param_header src/chimes_lsq.C:562-679
    const Controls& c = m.ctl;
    std::ostringstream h;
    h << "USECOUL: " << ((!c.fit_coul && !c.use_partial_charges) ? "false" : "true") << std::endl;
    h << "FITCOUL: " << (c.fit_coul ? "true" : "false") << std::endl;
    h << "USE3BCH: " << (c.use3 ? "true" : "false") << std::endl;
    h << "USE4BCH: " << (c.use4 ? "true" : "false") << std::endl;
    auto excl = [&](const char* tag, const std::vector<int>& v) {
        h << tag;
        if (v.empty()) h << "false";
        else for (int i : v) h << i << " ";
        h << std::endl;
    };
    excl("EXCLD1B: ", m.excl1b);
    excl("EXCLD2B: ", m.excl2b);
    const PairType& p0 = m.pairs[0];
    h << std::endl << "PAIRTYP: " << c.ff_type << " ";
    h << " " << p0.snum << " " << p0.snum3 << " " << p0.snum4 << " " << p0.range_low << " " << p0.range_high << std::endl;
    h << std::endl << "ATOM TYPES: " << c.natmtyp << std::endl << std::endl;
    h << "# TYPEIDX #\t# ATM_TYP #\t# ATMCHRG #\t# ATMMASS #" << std::endl;
    for (int i = 0; i < c.natmtyp; ++i) {   // FITCOUL prints the charge sign instead of the charge
        h << i << "\t\t" << m.pairs[i].atm1 << "\t\t";
        if (c.fit_coul) h << m.pairs[i].chrgsgn;
        else h << m.pairs[i].chg1;
        h << "\t\t" << m.pairs[i].mass1 << std::endl;
    }
    h << std::endl << "ATOM PAIRS: " << m.pairs.size() << std::endl << std::endl;
    h << "# PAIRIDX #\t# ATM_TY1 #\t# ATM_TY1 #\t# S_MINIM #\t# S_MAXIM #\t# CHBDIST #\t# MORSE_LAMBDA #" << std::endl;
    for (const auto& p : m.pairs) {
        h << "\t" << std::setw(16) << std::left << p.pairidx << std::setw(16) << std::left << p.atm1
          << std::setw(16) << std::left << p.atm2 << std::setw(16) << std::left << p.smin << std::setw(16)
          << std::left << p.smax << std::setw(16) << std::left << trans_string(p.trans);
        if (p.trans == TRANS_MORSE) h << std::setw(16) << std::left << p.lambda << std::endl;
        else h << std::endl;
    }
    h << std::endl << "FCUT TYPE: " << (c.fcut == FCUT_CUBIC ? "CUBIC" : "TERSOFF");
    if (c.fcut == FCUT_TERSOFF) h << " " << c.fcut_offset;
    h << std::endl;
    list_print_special(h, m.trips);
    list_print_special(h, m.quads);
    list_print_header(h, m.trips, 3, c.cheby3);
    list_print_header(h, m.quads, 4, c.cheby4);
    h << std::endl;
    return h.str();
}

std::string ff_groups_map_text(const Model& m) {   // print_map_file src/chimes_lsq.C:681-716
    std::ostringstream o;
    o << "PAIRMAPS: " << m.pair_map.size() << std::endl;
    for (const auto& kv : m.pair_map) o << kv.second << " " << kv.first << std::endl;
    if (!m.trips.map.empty()) {
        o << std::endl << "TRIPMAPS: " << m.trips.map.size() << std::endl;
        for (const auto& kv : m.trips.map) o << kv.second << " " << kv.first << std::endl;
    }
    if (!m.quads.map.empty()) {
        o << std::endl << "QUADMAPS: " << m.quads.map.size() << std::endl;
        for (const auto& kv : m.quads.map) o << kv.second << " " << kv.first << std::endl;
    }
    return o.str();
}

static std::string fmt(const char* f, ...) {
    char buf[256];
    va_list ap;
    va_start(ap, f);
    vsnprintf(buf, sizeof(buf), f, ap);
    va_end(ap);
    return buf;
}

static std::vector<std::string> split_lines(const std::string& t) {
    std::vector<std::string> out;
    std::stringstream ss(t);
    std::string l;
    while (std::getline(ss, l)) out.push_back(l);
    return out;
}

static std::vector<std::string> ws_split(const std::string& l) {   // python str.split()
    std::vector<std::string> t;
    std::stringstream ss(l);
    std::string w;
    while (ss >> w) t.push_back(w);
    return t;
}

static std::string rstrip_ws(std::string l) {
    while (!l.empty() && std::isspace((unsigned char)l.back())) l.pop_back();
    return l;
}

// The layout is driven by the params.header text, token by token, the way the
// solver script reads it back (src/chimes_lsq.py:316-672): header echo up to the
// TRIPLETS / QUADRUPLETS count lines, one "%3d %21.13e" line per 2-body power,
// the header's cluster power lines each followed by " %21.13e" of the coefficient
// named by its param-index column, ff_groups.map, then the energy offsets.
std::string params_txt_text(const Model& m, const double* x, int nx, const std::string& preamble) {
    if (nx != m.tot_all) throw Error(1, "coefficient count does not match the model's columns");
    std::ostringstream o;
    o << preamble;
    const std::vector<std::string> hf = split_lines(params_header_text(m));
    auto tok = [&](size_t line) {
        if (line >= hf.size()) throw Error(2, "params.header is shorter than its own counts");
        return ws_split(hf[line]);
    };
    auto at = [](const std::vector<std::string>& t, size_t i) -> const std::string& {
        if (i >= t.size()) throw Error(2, "params.header line has too few fields");
        return t[i];
    };
    size_t trip_line = 0, quad_line = 0;
    int ntrips = 0, nquads = 0;
    std::vector<int> excl1b, excl2b;   // EXCLD1B / EXCLD2B header lines (src/chimes_lsq.py:335-348)
    for (size_t i = 0; i < hf.size(); ++i) {
        o << hf[i] << "\n";
        const auto t = ws_split(hf[i]);
        bool done = false;
        for (int w = 0; w < 2; ++w) {
            if (hf[i].find(w == 0 ? "EXCLD2B" : "EXCLD1B") == std::string::npos) continue;
            std::vector<int>& ex = w == 0 ? excl2b : excl1b;
            ex.clear();
            if (!(t.size() == 2 && t[1] == "false"))
                for (size_t k = 1; k < t.size(); ++k) ex.push_back(std::stoi(t[k]));
        }
        if (t.size() > 3 && t[2] == "TRIPLETS:") {
            ntrips = std::stoi(t[3]);
            trip_line = i;
            for (size_t j = i; j < hf.size(); ++j) {
                const auto u = ws_split(hf[j]);
                if (u.size() > 3 && u[2] == "QUADRUPLETS:") {
                    o << hf[j] << "\n";
                    nquads = std::stoi(u[3]);
                    quad_line = j;
                    done = true;
                    break;
                }
            }
        }
        if (done) break;
    }
    const std::string potential = at(tok(7), 1);
    o << "\n" << "PAIR " << potential << " PARAMS \n\n";
    const auto pt = tok(7);
    const int snum = pt.size() >= 4 ? std::stoi(pt[2]) : 0;
    const size_t types_line = 9;
    const int ntypes = std::stoi(at(tok(types_line), 2));
    const size_t pairs_line = types_line + 2 + ntypes + 2;
    const int npairs = std::stoi(at(tok(pairs_line), 2));
    // FITCOUL: one "q_A x q_B" coefficient per pair after the short-range ones; the
    // short-range counts are read from the header as the solver script does
    // (src/chimes_lsq.py:394-458)
    const bool fit_coul = at(tok(1), 1) == "true";
    int snum3 = 0, snum4 = 0, counted_coul = 0;
    if (fit_coul) {
        auto count_unique = [&](size_t line0, int ncl, size_t uq, size_t tl) {
            int sum = 0, add = 0;
            for (int t = 0; t < ncl; ++t) {
                const auto p1 = tok(line0 + 3 + add);
                if (at(p1, uq) != "EXCLUDED:") {
                    sum += std::stoi(at(p1, uq));
                    add += 5 + std::stoi(at(p1, tl));
                }
            }
            return sum;
        };
        if (ntrips > 0) snum3 = count_unique(trip_line, ntrips, 4, 6);
        if (nquads > 0) snum4 = count_unique(quad_line, nquads, 7, 9);
    }
    int eff = 0;
    for (int i = 0; i < npairs; ++i) {
        const auto a = tok(pairs_line + 2 + i + 1);
        o << "PAIRTYPE PARAMS: " << i << " " << at(a, 1) << " " << at(a, 2) << "\n\n";
        if (std::find(excl2b.begin(), excl2b.end(), i) != excl2b.end()) {   // excluded: zeros
            for (int j = 0; j < snum; ++j) o << fmt("%3d %21.13e", j, 0.0) << "\n";
        } else {
            for (int j = 0; j < snum; ++j) o << fmt("%3d %21.13e", j, x[eff * snum + j]) << "\n";
            ++eff;
        }
        if (fit_coul) {
            const int col = npairs * snum + snum3 + snum4 + i;
            if (col >= nx) throw Error(2, "params.header names a charge coefficient out of range");
            o << "q_" << at(a, 1) << " x q_" << at(a, 2) << fmt(" %21.13e", x[col]) << "\n";
            ++counted_coul;
        }
        o << " \n";
    }
    // natoms 3: pair names in fields 1-3, counts in 4 / 6, power lines carry the param
    // index in column 5 (index, 3 powers, equiv, param);
    // natoms 4: pair names in fields 1-6, counts in 7 / 9, param index in column 8.
    int counted3 = 0, counted4 = 0;
    auto cluster_block = [&](size_t line0, int ncl, int natoms, int base) {
        const bool trip = natoms == 3;
        const size_t npn = trip ? 3 : 6;
        o << (trip ? "TRIPLET " : "QUADRUPLET ") << potential << " PARAMS \n\n";
        int add = 0, par = 0;
        for (int t = 0; t < ncl; ++t) {
            o << (trip ? "TRIPLETTYPE PARAMS:" : "QUADRUPLETYPE PARAMS: ") << "\n";
            o << "  " << rstrip_ws(hf.at(line0 + 2 + add)) << "\n";
            const auto p1 = tok(line0 + 3 + add);
            o << "   PAIRS:";
            for (size_t k = 1; k <= npn; ++k) o << " " << at(p1, k);
            if (at(p1, npn + 1) == "EXCLUDED:") {
                o << (trip ? " EXCLUDED:" : " EXCLUDED: ") << "\n";
                add += 1;
            } else {
                const int uniq = std::stoi(at(p1, npn + 1));
                const int totl = std::stoi(at(p1, npn + 3));
                o << " UNIQUE: " << at(p1, npn + 1) << " TOTAL: " << at(p1, npn + 3) << "\n";
                o << "     index  |  powers  |  equiv index  |  param index  |       parameter       \n";
                o << "   ----------------------------------------------------------------------------\n";
                add += 3;
                for (int p = 0; p < totl; ++p) {
                    add += 1;
                    const size_t ln = line0 + 2 + add;
                    const int pidx = std::stoi(at(tok(ln), npn + 2));
                    const int col = base + par + pidx;
                    if (col < 0 || col >= nx) throw Error(2, "params.header names a coefficient out of range");
                    o << hf[ln] << fmt(" %21.13e", x[col]) << "\n";
                }
                par += uniq;
                (trip ? counted3 : counted4) += uniq;
            }
            o << "\n";
            add += 2;
        }
    };
    if (ntrips > 0) cluster_block(trip_line, ntrips, 3, eff * snum);
    if (nquads > 0) cluster_block(quad_line, nquads, 4, eff * snum + counted3);
    o << "\n";
    for (const auto& l : split_lines(ff_groups_map_text(m))) o << l << "\n";
    o << "\n";
    const int total = eff * snum + counted3 + counted4 + counted_coul;
    const int n_offsets = ntypes - (int)excl1b.size();
    if (total != nx && nx != total + n_offsets) throw Error(2, "error in counting parameters");
    if (nx == total + n_offsets) {
        o << "NO ENERGY OFFSETS:  " << ntypes << "\n";
        int e = 0;
        for (int i = 0; i < ntypes; ++i) {
            const bool ex = std::find(excl1b.begin(), excl1b.end(), i) != excl1b.end();
            o << fmt("ENERGY OFFSET %d %21.13e", i + 1, ex ? 0.0 : x[total + e++]) << "\n";
        }
    }
    o << "ENDFILE\n";
    return o.str();
}

// ------------------------------------------------------------ box + frames

static double vec_mag(double a, double b, double c) {   // VECTOR_MAGNITUDE src/functions.C:47-56
    double mag = 0;
    mag += a * a; mag += b * b; mag += c * c;
    return std::sqrt(mag);
}
static double vec_angle(double a0, double a1, double a2, double b0, double b1, double b2) {   // :57-72
    double ang = 0;
    ang += a0 * b0; ang += a1 * b1; ang += a2 * b2;
    ang /= vec_mag(a0, a1, a2);
    ang /= vec_mag(b0, b1, b2);
    return std::acos(ang);
}

void constraint_rows(const Model& m, double* A, int64_t lda, double* b) {
    for (size_t i = 0; i < m.charge_constraints.size(); ++i) {
        const ChargeConstraint& cc = m.charge_constraints[i];
        double* row = A + (int64_t)i * lda;
        for (int c = 0; c < m.tot_all; ++c) row[c] = 0.0;
        for (size_t k = 0; k < cc.pair.size(); ++k) row[m.tot_short + cc.pair[k]] = cc.value[k];
        b[i] = cc.force;
    }
}

EwaldParams ewald_params(int natoms, const Box& box) {
    // Fincham, Mol. Sim. 1, 1-9 (1994): balance the real- and k-space errors at the
    // target accuracy; the same operations and constants as src/Ewald.C:428-475.
    const double accuracy = 1.0e-06, effort_ratio = 5.5, balance_factor = 1.1, accuracy_factor = 0.8;
    double min_boxdim = box.ax;
    if (box.by < min_boxdim) min_boxdim = box.by;
    if (box.cz < min_boxdim) min_boxdim = box.cz;
    const double V = box.ax * box.by * box.cz;
    const double p = -std::log(accuracy) * accuracy_factor;
    EwaldParams e;
    e.alpha = std::sqrt(M_PI) * std::pow(effort_ratio * natoms / (V * V), 1.0 / 6.0);
    e.rc = balance_factor * std::sqrt(p) / e.alpha;
    if (e.rc > 0.5 * min_boxdim) {
        e.rc = 0.5 * min_boxdim;
        e.alpha = std::sqrt(p) / e.rc;
    }
    const double rkc = 2.0 * e.alpha * std::sqrt(p) / balance_factor;
    const double lavg = std::pow(V, 1.0 / 3.0);
    e.kmax = (int)std::ceil(rkc * lavg / (2.0 * M_PI));
    return e;
}

void Box::update_cell() {   // BOX::UPDATE_CELL src/ClassDefs.C:1940-1971 (and the functions it calls)
    hmat[0] = ax; hmat[1] = bx; hmat[2] = cx;
    hmat[3] = ay; hmat[4] = by; hmat[5] = cy;
    hmat[6] = az; hmat[7] = bz; hmat[8] = cz;
    is_ortho = !(std::fabs(ay) + std::fabs(az) + std::fabs(bx) + std::fabs(bz) + std::fabs(cx) + std::fabs(cy) > 1.0e-10);
    // UPDATE_INVER_CELL src/ClassDefs.C:1776-1873
    const double* H = hmat;
    double det = H[0] * (H[4] * H[8] - H[5] * H[7]) - H[1] * (H[3] * H[8] - H[5] * H[6]) + H[2] * (H[3] * H[7] - H[4] * H[6]);
    if (det == 0) throw Error(2, "H-matrix determinant of zero");
    double T[9];
    T[0] = (H[4] * H[8] - H[5] * H[7]);
    T[1] = -1 * (H[3] * H[8] - H[5] * H[6]);
    T[2] = (H[3] * H[7] - H[4] * H[6]);
    T[3] = -1 * (H[1] * H[8] - H[2] * H[7]);
    T[4] = (H[0] * H[8] - H[2] * H[6]);
    T[5] = -1 * (H[0] * H[7] - H[1] * H[6]);
    T[6] = (H[1] * H[5] - H[2] * H[4]);
    T[7] = -1 * (H[0] * H[5] - H[2] * H[3]);
    T[8] = (H[0] * H[4] - H[1] * H[3]);
    invr[0] = T[0]; invr[1] = T[3]; invr[2] = T[6];
    invr[3] = T[1]; invr[4] = T[4]; invr[5] = T[7];
    invr[6] = T[2]; invr[7] = T[5]; invr[8] = T[8];
    for (int i = 0; i < 9; ++i) invr[i] /= det;
    // UPDATE_LAT_VALUES src/ClassDefs.C:1875-1897
    latcon_a = vec_mag(ax, ay, az);
    latcon_b = vec_mag(bx, by, bz);
    latcon_c = vec_mag(cx, cy, cz);
    alpha = vec_angle(bx, by, bz, cx, cy, cz);
    beta = vec_angle(cx, cy, cz, ax, ay, az);
    gamma = vec_angle(ax, ay, az, bx, by, bz);
    // LAMMPSIFY src/ClassDefs.C:1973-2021
    lx = latcon_a;
    xy = latcon_b * std::cos(gamma);
    if (std::fabs(xy) < 1e-12) xy = 0.0;
    xz = latcon_c * std::cos(beta);
    if (std::fabs(xz) < 1e-12) xz = 0.0;
    ly = std::sqrt(latcon_b * latcon_b - xy * xy);
    yz = (latcon_b * latcon_c * std::cos(alpha) - xy * xz) / ly;
    if (std::fabs(yz) < 1e-12) yz = 0.0;
    lz = std::sqrt(latcon_c * latcon_c - xz * xz - yz * yz);
    // UPDATE_EXTENT src/ClassDefs.C:1899-1938
    xlo = ylo = zlo = 0.0;
    if (xy < xlo) xlo = xy;
    if (xz < xlo) xlo = xz;
    if (xy + xz < xlo) xlo = xy + xz;
    if (yz < ylo) ylo = yz;
    xhi = ax;
    double tmp = 0.0;
    if (xy > tmp) tmp = xy;
    if (xz > tmp) tmp = xz;
    if (xy + xz > tmp) tmp = xy + xz;
    xhi += tmp;
    yhi = by;
    if (yz > 0.0) yhi += yz;
    zhi = cz;
    extent_x = xhi - xlo; extent_y = yhi - ylo; extent_z = zhi - zlo;
    // UPDATE_VOLUME src/ClassDefs.C:2193-2210
    if (is_ortho) vol = ax * by * cz;
    else {
        vol = 1;
        vol += 2 * std::cos(alpha) * std::cos(beta) * std::cos(gamma);
        vol -= std::cos(alpha) * std::cos(alpha);
        vol -= std::cos(beta) * std::cos(beta);
        vol -= std::cos(gamma) * std::cos(gamma);
        vol = latcon_a * latcon_b * latcon_c * std::sqrt(vol);
    }
}

// BOX::WRAP_ATOM src/ClassDefs.C:2075-2119 (in place)
void wrap_atom(const Box& b, double* x) {
    if (b.is_ortho) {
        int wx = (int)std::floor(x[0] / b.lx), wy = (int)std::floor(x[1] / b.ly), wz = (int)std::floor(x[2] / b.lz);
        x[0] = x[0] - wx * b.lx; x[1] = x[1] - wy * b.ly; x[2] = x[2] - wz * b.lz;
    } else {
        const double* I = b.invr;
        const double* H = b.hmat;
        double t0 = I[0] * x[0] + I[1] * x[1] + I[2] * x[2];
        double t1 = I[3] * x[0] + I[4] * x[1] + I[5] * x[2];
        double t2 = I[6] * x[0] + I[7] * x[1] + I[8] * x[2];
        int wx = (int)std::floor(t0), wy = (int)std::floor(t1), wz = (int)std::floor(t2);
        t0 -= wx; t1 -= wy; t2 -= wz;
        x[0] = H[0] * t0 + H[1] * t1 + H[2] * t2;
        x[1] = H[3] * t0 + H[4] * t1 + H[5] * t2;
        x[2] = H[6] * t0 + H[7] * t1 + H[8] * t2;
    }
}

std::vector<Frame> read_xyzf(const Model& m, const std::string& path, int nframes, int first_index, Box& box) {
    std::ifstream in(path);
    if (!in.is_open()) throw Error(2, "cannot open trajectory file: " + path);
    const Controls& c = m.ctl;
    std::vector<Frame> out;
    out.reserve(nframes);
    for (int f = 0; f < nframes; ++f) {
        const int fi = first_index + f;
        Frame fr;
        fr.index = fi;
        if (!(in >> fr.natoms)) throw Error(2, "unexpected end of trajectory at frame " + std::to_string(fi));
        std::string header;
        std::getline(in, header);
        std::getline(in, header);
        std::vector<std::string> tk;
        int nt = parse_space(header, tk);
        if (nt == 0) throw Error(2, "missing box line in frame " + std::to_string(fi));
        if (tk[0] == "NON_ORTHO") box.is_ortho = false;
        if (nt < 3) throw Error(2, "missing box length components in frame " + std::to_string(fi));
        if (box.is_ortho) {
            box.ax = to_double(tk[0]); box.by = to_double(tk[1]); box.cz = to_double(tk[2]);
        } else {
            if (nt < 10) throw Error(2, "NON_ORTHO box needs 9 components in frame " + std::to_string(fi));
            box.ax = to_double(tk[1]); box.ay = to_double(tk[2]); box.az = to_double(tk[3]);
            box.bx = to_double(tk[4]); box.by = to_double(tk[5]); box.bz = to_double(tk[6]);
            box.cx = to_double(tk[7]); box.cy = to_double(tk[8]); box.cz = to_double(tk[9]);
        }
        if (c.nstress < 0 || fi < c.nstress) {
            if (c.fit_stress) {
                if (box.is_ortho && nt >= 6) { for (int k = 0; k < 3; ++k) fr.stress_diag[k] = to_double(tk[3 + k]); }
                else if (!box.is_ortho && nt >= 13) { for (int k = 0; k < 3; ++k) fr.stress_diag[k] = to_double(tk[10 + k]); }
                else throw Error(2, "missing diagonal stress tensor components in frame " + std::to_string(fi));
            } else if (c.fit_stress_all) {
                int o = box.is_ortho ? 3 : 10;
                if (nt < o + 6) throw Error(2, "missing full stress tensor components in frame " + std::to_string(fi));
                for (int k = 0; k < 3; ++k) fr.stress_diag[k] = to_double(tk[o + k]);
                for (int k = 0; k < 3; ++k) fr.stress_off[k] = to_double(tk[o + 3 + k]);
            }
        }
        box.update_cell();
        if ((c.nener < 0 || fi < c.nener) && c.fit_ener) fr.energy = to_double(tk[nt - 1]);
        if (box.ax <= 0.0 || box.by <= 0.0 || box.cz <= 0.0) throw Error(2, "non-positive diagonal cell vector");
        if (std::fabs(box.ay) > 0.0 || std::fabs(box.az) > 0.0) throw Error(2, "A cell vector must be aligned on X axis");
        if (std::fabs(box.bz) > 0.0) throw Error(2, "B cell vector must be aligned in XY plane");
        fr.box = box;
        fr.type.resize(fr.natoms);
        fr.xyz.resize(3 * (size_t)fr.natoms);
        fr.force.resize(3 * (size_t)fr.natoms);
        for (int j = 0; j < fr.natoms; ++j) {
            std::string t;
            in >> t;
            size_t k = 0;
            for (; k < m.atom_types.size(); ++k) if (t == m.atom_types[k]) break;
            if (k == m.atom_types.size()) throw Error(2, "did not recognize atom type " + t);
            fr.type[j] = (int)k;
            double* x = &fr.xyz[3 * (size_t)j];
            double* fo = &fr.force[3 * (size_t)j];
            if (!(in >> x[0] >> x[1] >> x[2] >> fo[0] >> fo[1] >> fo[2]))
                throw Error(2, "truncated atom line in frame " + std::to_string(fi));
            for (int q = 0; q < 3; ++q) fo[q] *= FORCE_CONV;
            if (c.wrap) wrap_atom(fr.box, x);
        }
        out.push_back(std::move(fr));
    }
    return out;
}

std::vector<std::vector<int>> rank_frames(const Controls& c, int nprocs) {
    if (nprocs < 1) throw Error(1, "the rank count must be at least 1");
    std::vector<std::vector<int>> out(nprocs);
    const int n = c.nframes;
    for (int r = 0; r < nprocs; ++r) {
        if (c.skip_frames >= 1) {
            for (int i = 0; i < n; ++i)
                if ((i + r) % nprocs == 0 && ((i + r) / nprocs) % c.skip_frames == 0) out[r].push_back(i);
            continue;
        }
        if (n <= 0) continue;
        const int used = nprocs <= n ? nprocs : n;
        int beg = (int)std::ceil((double)r * n / used), end;
        if (r > n) { beg = n + 1; end = n - 1; }
        else if (r == used - 1) end = n - 1;
        else end = std::min((int)std::ceil((double)(r + 1) * n / used) - 1, n - 1);
        for (int i = beg; i <= end; ++i) out[r].push_back(i);
    }
    return out;
}

std::vector<Frame> read_frames(const Model& m, int nprocs) {
    // NFRAMES frames in file order (chimes_lsq.C:263-300: the next file opens when
    // a file's INFILE_FRAMES are used up); one SYSTEM box carries across files
    const Controls& c = m.ctl;
    if (c.infile.empty()) throw Error(2, "no TRJFILE given");
    Box box;
    std::vector<Frame> all;
    int done = 0;
    for (size_t k = 0; k < c.infile.size() && done < c.nframes; ++k) {
        std::string p = c.infile[k];
        if (!p.empty() && p[0] != '/') p = m.dir + "/" + p;
        const int n = std::min(c.nframes - done, k < c.infile_frames.size() ? c.infile_frames[k] : c.nframes - done);
        std::vector<Frame> part = read_xyzf(m, p, n, done, box);
        for (Frame& f : part) { f.file = (int)k; all.push_back(std::move(f)); }
        done += n;
    }
    if (done < c.nframes) throw Error(2, "the trajectory files hold fewer than NFRAMES frames");
    if (nprocs == 1 && c.skip_frames <= 0) return all;
    std::vector<Frame> out;
    const std::vector<std::vector<int>> sched = rank_frames(c, nprocs);
    for (int r = 0; r < nprocs; ++r)
        for (int i : sched[r]) { out.push_back(all[i]); out.back().rank = r; }
    return out;
}

RowLayout frame_rows(const Model& m, int fi, int natoms) {
    RowLayout r;
    r.force_rows = 3 * natoms;
    if (m.ctl.fit_stress && fi < m.ctl.nstress) r.stress_rows = 3;
    else if (m.ctl.fit_stress_all && fi < m.ctl.nstress) r.stress_rows = 9;
    if (m.ctl.fit_ener && fi < m.ctl.nener) r.energy_rows = 3;
    return r;
}

bool frame_is_small(const Model& m, const Box& b, bool previous_small) {
    if (previous_small || m.ctl.force_small || !m.ctl.use_neigh) return true;
    double mc = -1.0;   // NEIGHBORS::MAX_ALL_CUTOFFS src/ClassDefs.C:125-135
    if (m.max_cutoff_2b > mc) mc = m.max_cutoff_2b;
    if (m.max_cutoff_3b > mc) mc = m.max_cutoff_3b;
    if (m.max_cutoff_4b > mc) mc = m.max_cutoff_4b;
    return b.extent_x <= mc || b.extent_y <= mc || b.extent_z <= mc;
}

}  // namespace cg
