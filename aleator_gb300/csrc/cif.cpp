// CIF structure reader (host code): the framework input of the hot path.
//
// Reference: readCif (io/structure_io.hpp:51, io/structure_io.cc:177-245) over
// parseCifDocument (io/cif_document.cc:180-340), parseSymmetryOperation
// (io/symmetry_operation.cc:104-151) and the element table
// (io/element_table.cc). Same accepted grammar, the same error messages
// (with the line where the reference names one), the same species numbering
// (first appearance of each element), the same symmetry-orbit deduplication
// (images closer than 1e-3 A after a rounded fractional wrap) and the same
// IEEE operation order for the cell matrix and the Cartesian positions, so
// the particles equal the reference's bit for bit on the same host.
//
// Layout: a line cursor over the text, a per-line tokenizer, and one pass that
// fills a tag map and a list of loops; the structure is then assembled from
// them. Compiled with -ffp-contract=off (no fused multiply-adds).

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "common.cuh"
#include "cif.h"

namespace alea {

namespace {

[[noreturn]] void cif_fail(const std::string& msg) { throw Error(ALEA_ERR_RUNTIME, msg); }
[[noreturn]] void cif_fail_at(const std::string& msg, size_t line) {
    throw Error(ALEA_ERR_RUNTIME, msg + " (line " + std::to_string(line) + ")");
}

bool sp(char c) { return c == ' ' || c == '\t' || c == '\r'; }
char lower(char c) { return (char)std::tolower((unsigned char)c); }
std::string lowered(std::string s) {
    for (char& c : s) c = lower(c);
    return s;
}
bool blank(const std::string& s) {
    for (char c : s)
        if (!std::isspace((unsigned char)c)) return false;
    return true;
}
bool has_prefix_ci(const std::string& s, size_t at, const char* p) {
    for (size_t k = 0; p[k]; ++k)
        if (at + k >= s.size() || lower(s[at + k]) != p[k]) return false;
    return true;
}
size_t first_non_sp(const std::string& s) {
    size_t k = 0;
    while (k < s.size() && sp(s[k])) ++k;
    return k;
}

// Whitespace-separated fields of one line; a field opened by ' or " closes at
// the same quote followed by whitespace or the end of the line; an unquoted
// '#' comments out the rest of the line.
std::vector<std::string> fields(const std::string& s, size_t line) {
    std::vector<std::string> out;
    size_t i = 0;
    const size_t n = s.size();
    for (;;) {
        while (i < n && sp(s[i])) ++i;
        if (i >= n || s[i] == '#') return out;
        if (s[i] == '\'' || s[i] == '"') {
            const char q = s[i++];
            size_t j = i;
            while (j < n && !(s[j] == q && (j + 1 >= n || sp(s[j + 1])))) ++j;
            if (j >= n) cif_fail_at("unterminated quoted string", line);
            out.push_back(s.substr(i, j - i));
            i = j + 1;
        } else {
            size_t j = i;
            while (j < n && !sp(s[j]) && s[j] != '#') ++j;
            out.push_back(s.substr(i, j - i));
            i = j;
        }
    }
}

struct Loop {
    std::vector<std::string> cols;
    std::vector<std::vector<std::string>> rows;
    int col(const std::string& tag) const {
        for (size_t k = 0; k < cols.size(); ++k)
            if (cols[k] == tag) return (int)k;
        return -1;
    }
};

struct Doc {
    std::map<std::string, std::string> tags;  // lower-case tag -> raw value
    std::vector<Loop> loops;
    const std::string* tag(const char* t) const {
        const auto it = tags.find(t);
        return it == tags.end() ? nullptr : &it->second;
    }
    const Loop* loop_with(std::initializer_list<const char*> need) const {
        for (const Loop& l : loops) {
            bool all = true;
            for (const char* t : need) all = all && l.col(t) >= 0;
            if (all) return &l;
        }
        return nullptr;
    }
};

// The first data block of the text (parseCifDocument's grammar).
Doc parse_doc(const std::string& text) {
    std::vector<std::string> L;
    {
        size_t a = 0;
        for (;;) {
            const size_t b = text.find('\n', a);
            std::string s = text.substr(a, b == std::string::npos ? std::string::npos : b - a);
            if (!s.empty() && s.back() == '\r') s.pop_back();
            L.push_back(std::move(s));
            if (b == std::string::npos) break;
            a = b + 1;
        }
    }
    const size_t n = L.size();
    Doc d;
    bool seen_data = false;
    size_t i = 0;
    while (i < n) {
        const size_t ln = i + 1;
        if (blank(L[i])) {
            ++i;
            continue;
        }
        const size_t c0 = first_non_sp(L[i]);
        if (L[i][c0] == '#') {
            ++i;
            continue;
        }
        if (has_prefix_ci(L[i], c0, "data_")) {
            if (seen_data) break;  // later blocks are ignored
            (void)fields(L[i], ln);
            seen_data = true;
            ++i;
            continue;
        }
        if (has_prefix_ci(L[i], c0, "loop_")) {
            ++i;
            Loop lp;
            for (; i < n; ++i) {  // the column tags
                if (blank(L[i])) continue;
                const size_t k = first_non_sp(L[i]);
                if (k < L[i].size() && L[i][k] == '#') continue;
                if (k >= L[i].size() || L[i][k] != '_') break;
                const auto f = fields(L[i], i + 1);
                if (f.empty()) cif_fail_at("empty loop_ column declaration", i + 1);
                lp.cols.push_back(lowered(f[0]));
            }
            if (lp.cols.empty()) cif_fail_at("loop_ with no column declarations", ln);
            std::vector<std::string> row;
            size_t last = ln;
            for (; i < n; ++i) {  // values, rows spanning lines freely
                if (blank(L[i])) continue;
                if (row.empty()) {
                    const size_t k = first_non_sp(L[i]);
                    if (k < L[i].size() && L[i][k] != '#' &&
                        (L[i][k] == '_' || has_prefix_ci(L[i], k, "loop_") ||
                         has_prefix_ci(L[i], k, "data_")))
                        break;
                }
                last = i + 1;
                for (std::string& v : fields(L[i], i + 1)) {
                    row.push_back(std::move(v));
                    if (row.size() == lp.cols.size()) {
                        lp.rows.push_back(std::move(row));
                        row.clear();
                    }
                }
            }
            if (!row.empty())
                cif_fail_at("loop_ row has " + std::to_string(row.size()) + " value(s) but " +
                                std::to_string(lp.cols.size()) + " columns (" +
                                std::to_string(lp.cols.size() - row.size()) + " short)",
                            last);
            d.loops.push_back(std::move(lp));
            continue;
        }
        if (L[i][c0] == '_') {
            const auto f = fields(L[i], ln);
            const std::string tag = lowered(f[0]);
            std::string value;
            ++i;
            if (f.size() >= 2) {
                value = f[1];
            } else if (i < n && !L[i].empty() && L[i][0] == ';') {  // text field
                const size_t open = i + 1;
                std::vector<std::string> parts;
                if (L[i].size() > 1) parts.push_back(L[i].substr(1));
                bool closed = false;
                for (++i; i < n; ++i)
                    if (!L[i].empty() && L[i][0] == ';') {
                        closed = true;
                        ++i;
                        break;
                    } else {
                        parts.push_back(L[i]);
                    }
                if (!closed) cif_fail_at("unterminated ';' text field for tag " + tag, open);
                for (size_t k = 0; k < parts.size(); ++k) value += (k ? "\n" : "") + parts[k];
            } else if (i < n) {
                const auto v = fields(L[i], i + 1);
                if (v.empty()) cif_fail_at("missing value for tag " + tag, ln);
                value = v[0];
                ++i;
            } else {
                cif_fail_at("missing value for tag " + tag + " at end of file", ln);
            }
            d.tags[tag] = value;
            continue;
        }
        cif_fail_at("unrecognized content outside of a tag, loop_, or data_ block", ln);
    }
    if (!seen_data) cif_fail("no data_ block found in file");
    return d;
}

// A CIF number: "?" and "." are absent; a trailing "(esd)" is dropped; the
// rest must parse completely (tryParseCifNumber, cif_document.cc:152-178).
bool cif_number(const std::string& tok, double& out) {
    if (tok == "?" || tok == ".") return false;
    const std::string s = tok.substr(0, tok.find('('));
    if (s.empty()) return false;
    try {
        size_t used = 0;
        out = std::stod(s, &used);
        return used == s.size();
    } catch (const std::exception&) {
        return false;
    }
}
double need_number(const std::string& tok) {
    double v;
    if (!cif_number(tok, v)) cif_fail("expected a number but found \"" + tok + "\"");
    return v;
}

// One symmetry-equivalent position "x',y',z'" as rows of coefficients on
// x, y, z plus a translation.
struct SymOp {
    double m[3][3];
    double t[3];
};

SymOp parse_symop(const std::string& text) {
    std::string s;
    for (char c : text)
        if (!std::isspace((unsigned char)c)) s += c;
    std::vector<std::string> comp(1);
    for (char c : s) {
        if (c != ',') {
            comp.back() += c;
            continue;
        }
        if (comp.size() >= 3)
            cif_fail("symmetry operation \"" + text + "\" has more than 3 comma-separated components");
        comp.emplace_back();
    }
    if (comp.size() != 3)
        cif_fail("symmetry operation \"" + text + "\" must have exactly 3 components, found " +
                 std::to_string(comp.size()));
    SymOp op{};
    for (int r = 0; r < 3; ++r) {
        const std::string& e = comp[r];
        if (e.empty()) cif_fail("empty component in symmetry operation \"" + text + "\"");
        size_t i = 0;
        while (i < e.size()) {
            double sign = 1.0;
            if (e[i] == '+' || e[i] == '-') sign = e[i++] == '-' ? -1.0 : 1.0;
            if (i >= e.size()) cif_fail("trailing sign with no term in symmetry operation \"" + text + "\"");
            bool num = false;
            double value = 1.0;
            if (std::isdigit((unsigned char)e[i]) || e[i] == '.') {
                const size_t a = i;
                while (i < e.size() && (std::isdigit((unsigned char)e[i]) || e[i] == '.')) ++i;
                value = std::strtod(e.substr(a, i - a).c_str(), nullptr);
                if (i < e.size() && e[i] == '/') {
                    const size_t b = ++i;
                    while (i < e.size() && std::isdigit((unsigned char)e[i])) ++i;
                    if (i == b) cif_fail("malformed fraction in symmetry operation \"" + text + "\"");
                    value = value / std::strtod(e.substr(b, i - b).c_str(), nullptr);
                }
                num = true;
            }
            const char v = i < e.size() ? lower(e[i]) : 0;
            if (v == 'x' || v == 'y' || v == 'z') {
                op.m[r][v - 'x'] += sign * (num ? value : 1.0);
                ++i;
            } else if (num) {
                op.t[r] += sign * value;
            } else {
                cif_fail("expected x, y, z, or a number in symmetry operation \"" + text + "\"");
            }
        }
    }
    return op;
}

// Standard atomic weights of the elements the reference's table knows
// (io/element_table.cc): the set decides which labels resolve, the masses
// fill the particles' mass.
const char* const kElementWeights =
    "H 1.008 He 4.003 Li 6.94 Be 9.012 B 10.81 C 12.011 N 14.007 O 15.999 F 18.998 Ne 20.180 "
    "Na 22.990 Mg 24.305 Al 26.982 Si 28.085 P 30.974 S 32.06 Cl 35.45 Ar 39.948 K 39.098 "
    "Ca 40.078 Sc 44.956 Ti 47.867 V 50.942 Cr 51.996 Mn 54.938 Fe 55.845 Co 58.933 Ni 58.693 "
    "Cu 63.546 Zn 65.38 Ga 69.723 Ge 72.630 As 74.922 Se 78.971 Br 79.904 Kr 83.798 Rb 85.468 "
    "Sr 87.62 Y 88.906 Zr 91.224 Nb 92.906 Mo 95.95 Tc 98.0 Ru 101.07 Rh 102.906 Pd 106.42 "
    "Ag 107.868 Cd 112.414 In 114.818 Sn 118.710 Sb 121.760 Te 127.60 I 126.904 Xe 131.293 "
    "Cs 132.905 Ba 137.327 La 138.905 Ce 140.116 Pr 140.908 Nd 144.242 Pm 145.0 Sm 150.36 "
    "Eu 151.964 Gd 157.25 Tb 158.925 Dy 162.500 Ho 164.930 Er 167.259 Tm 168.934 Yb 173.045 "
    "Lu 174.967 Hf 178.49 Ta 180.948 W 183.84 Re 186.207 Os 190.23 Ir 192.217 Pt 195.084 "
    "Au 196.967 Hg 200.592 Tl 204.38 Pb 207.2 Bi 208.980";

const std::vector<std::pair<std::string, double>>& elements() {
    static const std::vector<std::pair<std::string, double>> table = [] {
        std::vector<std::pair<std::string, double>> t;
        std::istringstream in(kElementWeights);
        std::string sym, w;
        while (in >> sym >> w) t.emplace_back(sym, std::strtod(w.c_str(), nullptr));
        return t;
    }();
    return table;
}

bool element_mass(const std::string& sym, double& mass) {  // exact case
    for (const auto& e : elements())
        if (e.first == sym) {
            mass = e.second;
            return true;
        }
    return false;
}

// The element a label starts with: its leading letters, a two-letter symbol
// tried before a one-letter one, case-insensitively (elementFromLabel).
bool element_of(const std::string& label, std::string& out) {
    size_t letters = 0;
    while (letters < label.size() && std::isalpha((unsigned char)label[letters])) ++letters;
    for (size_t len = 2; len >= 1; --len) {
        if (letters < len) continue;
        for (const auto& e : elements())
            if (e.first.size() == len && lowered(e.first) == lowered(label.substr(0, len))) {
                out = e.first;
                return true;
            }
    }
    return false;
}

// Fractional to Cartesian with rows a_i of m (Lattice::fractionalToCartesian,
// core/geometry/lattice.cc:157-164): r_j = f0 a0_j + f1 a1_j + f2 a2_j.
void frac_to_cart(const double* m, const double* f, double* r) {
    for (int j = 0; j < 3; ++j) r[j] = f[0] * m[j] + f[1] * m[3 + j] + f[2] * m[6 + j];
}

// The cell from a, b, c, alpha, beta, gamma: a along x, b in the xy plane
// (structure_io.cc:53-98).
void cell_matrix(const Doc& d, double* m) {
    static const char* const kNames[6] = {"_cell_length_a", "_cell_length_b", "_cell_length_c",
                                          "_cell_angle_alpha", "_cell_angle_beta", "_cell_angle_gamma"};
    double v[6];
    for (int k = 0; k < 6; ++k) {
        const std::string* s = d.tag(kNames[k]);
        if (!s) cif_fail(std::string("missing required tag ") + kNames[k]);
        v[k] = need_number(*s);
    }
    for (int k = 0; k < 3; ++k)
        if (!(v[k] > 0.0))
            cif_fail(std::string(kNames[k]) + " must be positive, got " + std::to_string(v[k]));
    for (int k = 3; k < 6; ++k)
        if (!(v[k] > 0.0 && v[k] < 180.0))
            cif_fail(std::string(kNames[k]) + " must be strictly between 0 and 180 degrees, got " +
                     std::to_string(v[k]));
    const double rad = 3.14159265358979323846 / 180.0;
    const double ca = std::cos(v[3] * rad), cb = std::cos(v[4] * rad), cg = std::cos(v[5] * rad);
    const double sg = std::sin(v[5] * rad);
    const double c = v[2];
    const double cz2 = 1.0 - ca * ca - cb * cb - cg * cg + 2.0 * ca * cb * cg;
    if (cz2 < 0.0)
        cif_fail("cell angles alpha/beta/gamma do not describe a valid parallelepiped "
                 "(negative squared c-component)");
    const double rows[9] = {v[0], 0.0, 0.0, v[1] * cg, v[1] * sg, 0.0,
                            c * cb, c * (ca - cb * cg) / sg, c * std::sqrt(cz2) / sg};
    for (int k = 0; k < 9; ++k) m[k] = rows[k];
}

std::string read_file(const char* path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) cif_fail(std::string("could not open file: ") + path);
    std::ostringstream s;
    s << in.rdbuf();
    return s.str();
}

}  // namespace

Structure read_cif(const char* path) {
    const Doc d = parse_doc(read_file(path));
    Structure st;
    cell_matrix(d, st.m);

    std::vector<SymOp> ops;
    const char* op_tag = "_symmetry_equiv_pos_as_xyz";
    const Loop* ol = d.loop_with({op_tag});
    if (!ol) ol = d.loop_with({op_tag = "_space_group_symop_operation_xyz"});
    if (!ol) {
        ops.push_back(parse_symop("x,y,z"));  // P1
    } else {
        const int c = ol->col(op_tag);
        for (const auto& row : ol->rows) ops.push_back(parse_symop(row[c]));
        if (ops.empty())
            cif_fail(std::string("symmetry loop (") + op_tag + ") contains no operations");
    }

    const Loop* al = d.loop_with({"_atom_site_label", "_atom_site_fract_x", "_atom_site_fract_y",
                                  "_atom_site_fract_z"});
    if (!al) cif_fail("no _atom_site loop with a label and fractional x/y/z coordinates was found");
    const int c_lab = al->col("_atom_site_label"), c_typ = al->col("_atom_site_type_symbol");
    const int c_x = al->col("_atom_site_fract_x"), c_y = al->col("_atom_site_fract_y"),
              c_z = al->col("_atom_site_fract_z");
    const int c_occ = al->col("_atom_site_occupancy"), c_q = al->col("_atom_site_charge");

    for (const auto& row : al->rows) {
        const std::string& label = row[c_lab];
        std::string el;
        if (!((c_typ >= 0 && element_of(row[c_typ], el)) || element_of(label, el)))
            cif_fail("could not determine a chemical element for atom site \"" + label + "\"");
        double mass;
        if (!element_mass(el, mass))
            cif_fail("unknown element \"" + el + "\" (no atomic mass data) for atom site \"" + label + "\"");
        const double f[3] = {need_number(row[c_x]), need_number(row[c_y]), need_number(row[c_z])};
        double occ = 1.0, q = 0.0;
        if (c_occ >= 0 && !cif_number(row[c_occ], occ)) occ = 1.0;
        if (c_q >= 0 && !cif_number(row[c_q], q)) q = 0.0;
        uint32_t sid = 0;
        while (sid < st.symbols.size() && st.symbols[sid] != el) ++sid;
        if (sid == st.symbols.size()) st.symbols.push_back(el);

        // the orbit: every operation's image wrapped into [0, 1), kept unless
        // within 1e-3 A of an image already kept (special positions)
        std::vector<std::array<double, 3>> orbit;
        for (const SymOp& op : ops) {
            std::array<double, 3> g;
            for (int r = 0; r < 3; ++r) {
                g[r] = op.m[r][0] * f[0] + op.m[r][1] * f[1] + op.m[r][2] * f[2] + op.t[r];
                g[r] -= std::floor(g[r]);
            }
            bool dup = false;
            for (const auto& o : orbit) {
                double dfr[3], dc[3];
                for (int r = 0; r < 3; ++r) {
                    dfr[r] = g[r] - o[r];
                    dfr[r] -= std::round(dfr[r]);
                }
                frac_to_cart(st.m, dfr, dc);
                if (std::sqrt(dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2]) < 1e-3) {
                    dup = true;
                    break;
                }
            }
            if (!dup) orbit.push_back(g);
        }
        for (const auto& g : orbit) {
            double r[3];
            frac_to_cart(st.m, g.data(), r);
            st.x.push_back(r[0]);
            st.y.push_back(r[1]);
            st.z.push_back(r[2]);
            st.charge.push_back(q);
            st.mass.push_back(mass);
            st.species.push_back(sid);
            st.occupancy.push_back(occ);
            st.labels.push_back(label);
        }
    }
    return st;
}

}  // namespace alea
