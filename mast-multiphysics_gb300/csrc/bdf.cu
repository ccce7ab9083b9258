// bdf.cu -- Nastran bulk data (BDF) mesh input, host code.
//
// The reference reads BDF files through pyNastran (MAST::NastranIO::read,
// src/mesh/nastran_io.cpp:221-339): GRID points become mesh nodes under their
// Nastran ids (read_nodes :105-125), CHEXA / CQUAD4 cards become HEX8 / QUAD4
// elements with the card's node order, which is libMesh's local order
// (read_elements :128-198), and every SPC node set becomes a node boundary
// (read_node_boundaries :201-218).  This reader is written from the bulk data
// format itself, without pyNastran: small-field (8-column), large-field
// (16-column, `NAME*`) and free-field (comma-separated) cards with continuation
// lines; GRID, CHEXA (8 nodes), CQUAD4, SPC1 (including `THRU`), SPC and FORCE.
// Nodes are numbered in ascending GRID id and elements in ascending element id;
// constraints and loads of every set id are taken (one load case), as the
// reference takes every SPC set.  Material and property cards are not read:
// the material comes from mg_material_desc.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <set>
#include <string>
#include <vector>

#include "mg_internal.h"

struct mg_bdf_mesh {
    std::vector<int64_t> node_ids;       // ascending GRID ids
    std::vector<double> coords;          // 3 per node
    int32_t npe = 0;                     // 8 (CHEXA) or 4 (CQUAD4)
    std::vector<int64_t> elem_ids;       // ascending element ids
    std::vector<int32_t> pids;
    std::vector<int32_t> conn;           // npe per element, node indices
    std::map<int64_t, int> spc;          // node index -> component bits (bit c-1 for component c)
    std::map<std::pair<int64_t, int>, double> force;  // (node index, component 0..2) -> force
};

namespace mg {
namespace {

std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) a++;
    while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

std::string upper(std::string s) {
    for (auto &ch : s) ch = (char)std::toupper((unsigned char)ch);
    return s;
}

// Nastran real: "1.5", "-2.", ".5E-1", "1.0D-3" and the exponent shorthand
// "1.5-3" (= 1.5e-3), "-2.5+2"; false if the field is not a number
bool parse_real(const std::string &f, double &out) {
    std::string s = upper(trim(f));
    if (s.empty()) return false;
    for (auto &ch : s)
        if (ch == 'D') ch = 'E';
    if (s.find('E') == std::string::npos) {
        // an inner sign after the mantissa starts the exponent
        for (size_t i = 1; i < s.size(); i++)
            if ((s[i] == '+' || s[i] == '-') && s[i - 1] != 'E') {
                s.insert(i, "E");
                break;
            }
    }
    char *end = nullptr;
    out = std::strtod(s.c_str(), &end);
    return end && *end == '\0';
}

bool parse_int(const std::string &f, int64_t &out) {
    std::string s = trim(f);
    if (s.empty()) return false;
    char *end = nullptr;
    out = std::strtoll(s.c_str(), &end, 10);
    return end && *end == '\0';
}

// one bulk data card: its name and data fields (fields 2.. of every line, the
// continuation markers dropped)
struct Card {
    std::string name;
    std::vector<std::string> f;
    int line = 0;
};

bool is_free(const std::string &line) { return line.find(',') != std::string::npos; }

// split a line into (first field, data fields)
void split_line(const std::string &raw, std::string &first, std::vector<std::string> &data) {
    data.clear();
    std::string line = raw;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    if (is_free(line)) {
        std::vector<std::string> parts;
        size_t start = 0;
        for (size_t i = 0; i <= line.size(); i++)
            if (i == line.size() || line[i] == ',') {
                parts.push_back(trim(line.substr(start, i - start)));
                start = i + 1;
            }
        first = parts.empty() ? "" : parts[0];
        // free field: up to 8 data fields per line, a 10th field is the continuation id
        for (size_t i = 1; i < parts.size() && i <= 8; i++) data.push_back(parts[i]);
        return;
    }
    auto field = [&](size_t col, size_t width) {
        return col < line.size() ? line.substr(col, std::min(width, line.size() - col)) : std::string();
    };
    first = trim(field(0, 8));
    const bool large = !first.empty() && (first.back() == '*' || first[0] == '*');
    if (large)
        for (int i = 0; i < 4; i++) data.push_back(trim(field(8 + 16 * i, 16)));
    else
        for (int i = 0; i < 8; i++) data.push_back(trim(field(8 + 8 * i, 8)));
}

bool parse_cards(const std::string &text, std::vector<Card> &cards, std::string &err) {
    std::vector<std::string> lines;
    size_t start = 0;
    for (size_t i = 0; i <= text.size(); i++)
        if (i == text.size() || text[i] == '\n') {
            lines.push_back(text.substr(start, i - start));
            start = i + 1;
        }
    // the bulk data section, if the file has one
    size_t lo = 0, hi = lines.size();
    for (size_t i = 0; i < lines.size(); i++)
        if (upper(trim(lines[i])).rfind("BEGIN BULK", 0) == 0) { lo = i + 1; break; }
    for (size_t i = lo; i < lines.size(); i++)
        if (upper(trim(lines[i])).rfind("ENDDATA", 0) == 0) { hi = i; break; }
    std::string first;
    std::vector<std::string> data;
    for (size_t i = lo; i < hi; i++) {
        const std::string t = trim(lines[i]);
        if (t.empty() || t[0] == '$') continue;
        split_line(lines[i], first, data);
        const bool cont = first.empty() || first[0] == '+' || first[0] == '*';
        if (cont) {
            if (cards.empty()) {
                err = "continuation line " + std::to_string(i + 1) + " without a card";
                return false;
            }
            for (auto &d : data) cards.back().f.push_back(d);
            continue;
        }
        Card c;
        c.name = upper(first);
        if (!c.name.empty() && c.name.back() == '*') c.name.pop_back();
        c.f = data;
        c.line = (int)i + 1;
        cards.push_back(c);
    }
    return true;
}

// a card's data fields without the trailing blanks
std::vector<std::string> used(const Card &c) {
    std::vector<std::string> f = c.f;
    while (!f.empty() && f.back().empty()) f.pop_back();
    return f;
}

int build_mesh(const std::vector<Card> &cards, mg_bdf_mesh &m) {
    auto bad = [&](const Card &c, const char *why) {
        set_error("BDF line %d (%s): %s", c.line, c.name.c_str(), why);
        return MG_EINVAL;
    };
    std::map<int64_t, std::array<double, 3>> grids;
    struct E { int64_t pid; std::vector<int64_t> g; int npe; int line; };
    std::map<int64_t, E> elems;
    std::vector<std::pair<int64_t, int>> spc_nodes;  // (GRID id, component digits)
    std::set<std::pair<int64_t, int>> spc_optional;  // from THRU ranges: ids that need not exist
    std::vector<std::pair<int64_t, std::array<double, 3>>> forces;
    for (const Card &c : cards) {
        const std::vector<std::string> f = used(c);
        if (c.name == "GRID") {
            int64_t id, cp = 0;
            double x[3];
            if (f.size() < 5 || !parse_int(f[0], id)) return bad(c, "GRID needs an id and x, y, z");
            if (!f[1].empty() && (!parse_int(f[1], cp) || cp != 0)) return bad(c, "only the basic coordinate system");
            for (int k = 0; k < 3; k++)
                if (!parse_real(f[2 + k], x[k])) return bad(c, "bad coordinate");
            if (grids.count(id)) return bad(c, "duplicate GRID id");
            grids[id] = {x[0], x[1], x[2]};
        } else if (c.name == "CHEXA" || c.name == "CQUAD4") {
            const int npe = c.name == "CHEXA" ? 8 : 4;
            int64_t eid, pid;
            if ((int)f.size() < 2 + npe || !parse_int(f[0], eid) || !parse_int(f[1], pid))
                return bad(c, "element needs an id, a property id and its nodes");
            E e{pid, {}, npe, c.line};
            for (int k = 0; k < npe; k++) {
                int64_t g;
                if (!parse_int(f[2 + k], g)) return bad(c, "bad node id");
                e.g.push_back(g);
            }
            if (c.name == "CHEXA" && f.size() > 10) return bad(c, "only 8-node CHEXA");
            if (elems.count(eid)) return bad(c, "duplicate element id");
            elems[eid] = e;
        } else if (c.name == "SPC1") {
            int64_t comp;
            if (f.size() < 3 || !parse_int(f[1], comp)) return bad(c, "SPC1 needs components and nodes");
            if (f.size() == 5 && upper(f[3]) == "THRU") {
                int64_t a, b;
                if (!parse_int(f[2], a) || !parse_int(f[4], b) || b < a) return bad(c, "bad THRU range");
                // the points of a THRU range need not all exist (the absent are skipped)
                for (int64_t g = a; g <= b; g++) {
                    spc_nodes.push_back({g, (int)comp});
                    spc_optional.insert({g, (int)comp});
                }
            } else {
                for (size_t k = 2; k < f.size(); k++) {
                    if (f[k].empty()) continue;
                    int64_t g;
                    if (!parse_int(f[k], g)) return bad(c, "bad node id");
                    spc_nodes.push_back({g, (int)comp});
                }
            }
        } else if (c.name == "SPC") {
            // SID, then (G, C, D) triples; only homogeneous constraints
            for (size_t k = 1; k + 1 < f.size(); k += 3) {
                int64_t g, comp;
                if (f[k].empty()) continue;
                if (!parse_int(f[k], g) || !parse_int(f[k + 1], comp)) return bad(c, "bad node or component");
                double d = 0.0;
                if (k + 2 < f.size() && !f[k + 2].empty() && (!parse_real(f[k + 2], d) || d != 0.0))
                    return bad(c, "only homogeneous SPC (D = 0)");
                spc_nodes.push_back({g, (int)comp});
            }
        } else if (c.name == "FORCE") {
            int64_t g, cid = 0;
            double s, n[3] = {0, 0, 0};
            if (f.size() < 4 || !parse_int(f[1], g) || !parse_real(f[3], s)) return bad(c, "FORCE needs G, CID, F, N");
            if (!f[2].empty() && (!parse_int(f[2], cid) || cid != 0)) return bad(c, "only the basic coordinate system");
            for (int k = 0; k < 3; k++)
                if (4 + k < (int)f.size() && !f[4 + k].empty() && !parse_real(f[4 + k], n[k])) return bad(c, "bad direction");
            forces.push_back({g, {s * n[0], s * n[1], s * n[2]}});
        }
        // other cards (properties, materials, case control leftovers) are not read
    }
    if (grids.empty() || elems.empty()) {
        set_error("BDF: no GRID or no CHEXA / CQUAD4 cards");
        return MG_EINVAL;
    }
    std::map<int64_t, int64_t> index;  // GRID id -> node index
    for (auto &kv : grids) {
        index[kv.first] = (int64_t)m.node_ids.size();
        m.node_ids.push_back(kv.first);
        for (int k = 0; k < 3; k++) m.coords.push_back(kv.second[k]);
    }
    m.npe = elems.begin()->second.npe;
    for (auto &kv : elems) {
        const E &e = kv.second;
        if (e.npe != m.npe) {
            set_error("BDF line %d: CHEXA and CQUAD4 in one mesh", e.line);
            return MG_EINVAL;
        }
        m.elem_ids.push_back(kv.first);
        m.pids.push_back((int32_t)e.pid);
        for (int64_t g : e.g) {
            auto it = index.find(g);
            if (it == index.end()) {
                set_error("BDF line %d: element %lld uses undefined GRID %lld", e.line, (long long)kv.first,
                          (long long)g);
                return MG_EINVAL;
            }
            m.conn.push_back((int32_t)it->second);
        }
    }
    for (auto &sc : spc_nodes) {
        auto it = index.find(sc.first);
        if (it == index.end()) {
            if (spc_optional.count(sc)) continue;
            set_error("BDF: SPC on undefined GRID %lld", (long long)sc.first);
            return MG_EINVAL;
        }
        int bits = 0;
        for (int64_t c = sc.second; c > 0; c /= 10) {
            const int d = (int)(c % 10);
            if (d < 1 || d > 6) {
                set_error("BDF: bad SPC component digit %d", d);
                return MG_EINVAL;
            }
            bits |= 1 << (d - 1);
        }
        m.spc[it->second] |= bits;
    }
    for (auto &fo : forces) {
        auto it = index.find(fo.first);
        if (it == index.end()) {
            set_error("BDF: FORCE on undefined GRID %lld", (long long)fo.first);
            return MG_EINVAL;
        }
        for (int k = 0; k < 3; k++)
            if (fo.second[k] != 0.0) m.force[{it->second, k}] += fo.second[k];
    }
    return MG_OK;
}

int parse_into(const std::string &text, mg_bdf_mesh **out) {
    // a deck larger than host memory allows comes back as MG_ENOMEM
    try {
        std::vector<Card> cards;
        std::string err;
        if (!parse_cards(text, cards, err)) {
            set_error("BDF: %s", err.c_str());
            return MG_EINVAL;
        }
        std::unique_ptr<mg_bdf_mesh> m(new mg_bdf_mesh());
        const int rc = build_mesh(cards, *m);
        if (rc != MG_OK) return rc;
        *out = m.release();
        return MG_OK;
    } catch (const std::bad_alloc &) {
        set_error("BDF: out of host memory");
        return MG_ENOMEM;
    }
}

}  // namespace
}  // namespace mg

using namespace mg;

extern "C" {

int mg_bdf_parse(const char *text, int64_t len, mg_bdf_mesh **out) {
    if (!text || len < 0 || !out) return MG_EINVAL;
    *out = nullptr;
    try {
        return parse_into(std::string(text, (size_t)len), out);
    } catch (const std::bad_alloc &) {
        set_error("BDF: out of host memory");
        return MG_ENOMEM;
    }
}

int mg_bdf_read(const char *path, mg_bdf_mesh **out) {
    if (!path || !out) return MG_EINVAL;
    *out = nullptr;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) {
        set_error("BDF: cannot open %s", path);
        return MG_EINVAL;
    }
    std::string text;
    char buf[1 << 16];
    size_t n;
    try {
        while ((n = std::fread(buf, 1, sizeof(buf), fp)) > 0) text.append(buf, n);
    } catch (const std::bad_alloc &) {
        std::fclose(fp);
        set_error("BDF: out of host memory");
        return MG_ENOMEM;
    }
    std::fclose(fp);
    return parse_into(text, out);
}

int mg_bdf_sizes(const mg_bdf_mesh *m, int64_t *n_nodes, int64_t *n_elems, int32_t *nodes_per_elem) {
    if (!m) return MG_EINVAL;
    if (n_nodes) *n_nodes = (int64_t)m->node_ids.size();
    if (n_elems) *n_elems = (int64_t)m->elem_ids.size();
    if (nodes_per_elem) *nodes_per_elem = m->npe;
    return MG_OK;
}

int mg_bdf_nodes(const mg_bdf_mesh *m, double *coords, int64_t *grid_ids) {
    if (!m) return MG_EINVAL;
    if (coords) std::memcpy(coords, m->coords.data(), m->coords.size() * sizeof(double));
    if (grid_ids) std::memcpy(grid_ids, m->node_ids.data(), m->node_ids.size() * sizeof(int64_t));
    return MG_OK;
}

int mg_bdf_elements(const mg_bdf_mesh *m, int32_t *conn, int64_t *elem_ids, int32_t *pids) {
    if (!m) return MG_EINVAL;
    if (conn) std::memcpy(conn, m->conn.data(), m->conn.size() * sizeof(int32_t));
    if (elem_ids) std::memcpy(elem_ids, m->elem_ids.data(), m->elem_ids.size() * sizeof(int64_t));
    if (pids) std::memcpy(pids, m->pids.data(), m->pids.size() * sizeof(int32_t));
    return MG_OK;
}

int mg_bdf_constraints(const mg_bdf_mesh *m, int32_t dpn, int64_t *fixed_dofs, int64_t *n) {
    if (!m || !n || dpn < 1 || dpn > 6) return MG_EINVAL;
    int64_t k = 0;
    for (auto &kv : m->spc)
        for (int c = 0; c < dpn; c++)
            if ((kv.second >> c) & 1) {
                if (fixed_dofs) fixed_dofs[k] = (int64_t)dpn * kv.first + c;
                k++;
            }
    *n = k;
    return MG_OK;
}

int mg_bdf_loads(const mg_bdf_mesh *m, int32_t dpn, int64_t *load_dofs, double *load_values, int64_t *n) {
    if (!m || !n || dpn < 1) return MG_EINVAL;
    int64_t k = 0;
    for (auto &kv : m->force) {
        if (kv.first.second >= dpn) continue;
        if (load_dofs) load_dofs[k] = (int64_t)dpn * kv.first.first + kv.first.second;
        if (load_values) load_values[k] = kv.second;
        k++;
    }
    *n = k;
    return MG_OK;
}

void mg_bdf_destroy(mg_bdf_mesh *m) { delete m; }

}  // extern "C"
