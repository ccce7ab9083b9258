// exodus.cu -- ExodusII files, host code.
//
// MAST writes its solutions (displacements, densities, mode shapes) through
// libMesh's ExodusII_IO (examples/structural/example_7/example_7.cpp:256-281,
// write_timestep), and its structured and imported meshes can come from ExodusII
// files.  This is an ExodusII reader and writer written from the two public
// format descriptions, without the Exodus or netCDF libraries:
//   * the netCDF classic file format (CDF-1: 32-bit offsets, CDF-2: 64-bit
//     offsets): magic "CDF" + version byte, number of records, then the
//     dimension, global attribute and variable lists (tags 10, 12, 11), every
//     integer big-endian, names and values padded to four bytes; fixed-size
//     variables stored at their begin offsets, record variables interleaved one
//     record after another;
//   * the ExodusII data model on top of it: num_dim / num_nodes / num_elem /
//     num_el_blk, coordx..coordz (or coord), connect<b> with its elem_type
//     attribute (1-based node numbers), time_whole, vals_nod_var<i> and
//     vals_elem_var<i>eb<b> over the time_step record dimension with their
//     name tables.
// The writer emits CDF-2 with one element block and one time step; the reader
// takes CDF-1 or CDF-2 (not netCDF-4 / HDF5) with any number of blocks of one
// element type (HEX8 or QUAD4 families), concatenated in block order.
#include <algorithm>
#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "mg_internal.h"

namespace mg {
namespace {

enum : uint32_t { kNcByte = 1, kNcChar = 2, kNcShort = 3, kNcInt = 4, kNcFloat = 5, kNcDouble = 6 };
enum : uint32_t { kTagDim = 10, kTagVar = 11, kTagAtt = 12 };

int type_size(uint32_t t) {
    switch (t) {
        case kNcByte: case kNcChar: return 1;
        case kNcShort: return 2;
        case kNcInt: case kNcFloat: return 4;
        case kNcDouble: return 8;
        default: return 0;
    }
}

// ---------------------------------------------------------------- writer
struct Buf {
    std::vector<uint8_t> b;
    void u32(uint32_t v) {
        for (int s = 24; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
    }
    void u64(uint64_t v) {
        for (int s = 56; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
    }
    void f64(double d) {
        uint64_t v;
        memcpy(&v, &d, 8);
        u64(v);
    }
    void pad4() {
        while (b.size() % 4) b.push_back(0);
    }
    void name(const std::string &s) {
        u32((uint32_t)s.size());
        b.insert(b.end(), s.begin(), s.end());
        pad4();
    }
};

struct WAtt {
    std::string name;
    uint32_t type;
    std::vector<uint8_t> raw;  // big-endian values
    uint32_t n;
};
WAtt att_text(const std::string &name, const std::string &v) {
    return WAtt{name, kNcChar, std::vector<uint8_t>(v.begin(), v.end()), (uint32_t)v.size()};
}
WAtt att_int(const std::string &name, int32_t v) {
    Buf t;
    t.u32((uint32_t)v);
    return WAtt{name, kNcInt, t.b, 1};
}
WAtt att_float(const std::string &name, float v) {
    uint32_t u;
    memcpy(&u, &v, 4);
    Buf t;
    t.u32(u);
    return WAtt{name, kNcFloat, t.b, 1};
}

struct WVar {
    std::string name;
    std::vector<int> dims;
    std::vector<WAtt> atts;
    uint32_t type;
    std::vector<uint8_t> data;  // big-endian, one record's worth for record variables
    bool record;
};

void put_atts(Buf &h, const std::vector<WAtt> &atts) {
    if (atts.empty()) {
        h.u32(0);
        h.u32(0);
        return;
    }
    h.u32(kTagAtt);
    h.u32((uint32_t)atts.size());
    for (const WAtt &a : atts) {
        h.name(a.name);
        h.u32(a.type);
        h.u32(a.n);
        h.b.insert(h.b.end(), a.raw.begin(), a.raw.end());
        h.pad4();
    }
}

std::vector<uint8_t> be_doubles(const double *v, int64_t n) {
    Buf t;
    t.b.reserve((size_t)n * 8);
    for (int64_t i = 0; i < n; i++) t.f64(v[i]);
    return t.b;
}
std::vector<uint8_t> be_ints(const std::vector<int32_t> &v) {
    Buf t;
    t.b.reserve(v.size() * 4);
    for (int32_t x : v) t.u32((uint32_t)x);
    return t.b;
}
std::vector<uint8_t> name_table(const std::vector<std::string> &names, int len) {
    std::vector<uint8_t> out((size_t)names.size() * len, 0);
    for (size_t i = 0; i < names.size(); i++)
        memcpy(out.data() + i * len, names[i].data(), std::min<size_t>(names[i].size(), (size_t)len - 1));
    return out;
}

// ---------------------------------------------------------------- reader
struct RVar {
    std::vector<uint32_t> dims;
    std::map<std::string, std::string> text_atts;
    uint32_t type = 0;
    uint64_t vsize = 0, begin = 0;
};
struct NcFile {
    std::vector<uint8_t> raw;
    int version = 0;
    uint64_t numrecs = 0, recsize = 0;
    std::vector<std::pair<std::string, uint64_t>> dims;  // length 0 = the record dimension
    std::map<std::string, RVar> vars;
    int record_dim = -1;

    size_t pos = 0;
    bool ok = true;
    uint32_t u32() {
        if (pos + 4 > raw.size()) { ok = false; return 0; }
        const uint32_t v = ((uint32_t)raw[pos] << 24) | ((uint32_t)raw[pos + 1] << 16) |
                           ((uint32_t)raw[pos + 2] << 8) | raw[pos + 3];
        pos += 4;
        return v;
    }
    uint64_t u64() {
        const uint64_t hi = u32();
        return (hi << 32) | u32();
    }
    std::string name() {
        const uint32_t n = u32();
        if (!ok || pos + n > raw.size()) { ok = false; return ""; }
        std::string s(reinterpret_cast<const char *>(raw.data() + pos), n);
        pos += (n + 3) & ~3u;
        return s;
    }
    std::map<std::string, std::string> atts() {
        std::map<std::string, std::string> out;
        const uint32_t tag = u32(), n = u32();
        if (tag == 0) return out;
        if (tag != kTagAtt) { ok = false; return out; }
        for (uint32_t i = 0; i < n && ok; i++) {
            const std::string nm = name();
            const uint32_t t = u32(), cnt = u32();
            const uint64_t bytes = (uint64_t)cnt * type_size(t);
            if (pos + bytes > raw.size() || type_size(t) == 0) { ok = false; break; }
            if (t == kNcChar) {
                std::string v(reinterpret_cast<const char *>(raw.data() + pos), (size_t)bytes);
                while (!v.empty() && v.back() == '\0') v.pop_back();
                out[nm] = v;
            }
            pos += (bytes + 3) & ~(uint64_t)3;
        }
        return out;
    }
    bool parse() {
        if (raw.size() < 8 || raw[0] != 'C' || raw[1] != 'D' || raw[2] != 'F') return false;
        version = raw[3];
        if (version != 1 && version != 2) return false;
        pos = 4;
        numrecs = u32();
        uint32_t tag = u32(), n = u32();
        if (tag == kTagDim)
            for (uint32_t i = 0; i < n && ok; i++) {
                const std::string nm = name();
                const uint64_t len = u32();
                if (len == 0) record_dim = (int)dims.size();
                dims.push_back({nm, len});
            }
        else if (tag != 0) return false;
        atts();  // global attributes
        tag = u32();
        n = u32();
        if (tag == kTagVar)
            for (uint32_t i = 0; i < n && ok; i++) {
                const std::string nm = name();
                RVar v;
                const uint32_t nd = u32();
                for (uint32_t k = 0; k < nd && ok; k++) {
                    const uint32_t id = u32();
                    if (id >= dims.size()) { ok = false; break; }
                    v.dims.push_back(id);
                }
                v.text_atts = atts();
                v.type = u32();
                v.vsize = u32();
                v.begin = version == 1 ? u32() : u64();
                if (!v.dims.empty() && (int)v.dims[0] == record_dim) recsize += v.vsize;
                vars[nm] = v;
            }
        else if (tag != 0) return false;
        return ok;
    }
    bool has(const std::string &nm) const { return vars.count(nm) != 0; }
    uint64_t dim_len(const std::string &nm) const {
        for (const auto &d : dims)
            if (d.first == nm) return d.second;
        return 0;
    }
    // the values of a fixed-size numeric variable (record variables: record `rec`) as doubles
    bool values(const std::string &nm, std::vector<double> &out, uint64_t rec = 0) const {
        auto it = vars.find(nm);
        if (it == vars.end()) return false;
        const RVar &v = it->second;
        const int ts = type_size(v.type);
        if (ts == 0 || v.type == kNcChar) return false;
        // every size is checked against the file before it is multiplied or added, so
        // that no header value can wrap an offset past the end of the data
        const uint64_t limit = raw.size() / (uint64_t)ts;
        uint64_t count = 1;
        bool is_rec = false;
        for (size_t k = 0; k < v.dims.size(); k++) {
            if ((int)v.dims[k] == record_dim && k == 0) { is_rec = true; continue; }
            const uint64_t len = dims[v.dims[k]].second;
            if (len != 0 && count > limit / len) return false;
            count *= len;
        }
        if (v.begin > raw.size() || (is_rec && recsize != 0 && rec > (raw.size() - v.begin) / recsize))
            return false;
        const uint64_t start = v.begin + (is_rec ? rec * recsize : 0);
        if (start > raw.size() || count > (raw.size() - start) / (uint64_t)ts) return false;
        out.resize((size_t)count);
        const uint8_t *p = raw.data() + start;
        for (uint64_t i = 0; i < count; i++, p += ts) {
            uint64_t u = 0;
            for (int b = 0; b < ts; b++) u = (u << 8) | p[b];
            switch (v.type) {
                case kNcByte: out[i] = (double)(int8_t)u; break;
                case kNcShort: out[i] = (double)(int16_t)u; break;
                case kNcInt: out[i] = (double)(int32_t)(uint32_t)u; break;
                case kNcFloat: { uint32_t w = (uint32_t)u; float f; memcpy(&f, &w, 4); out[i] = f; break; }
                default: { double d; memcpy(&d, &u, 8); out[i] = d; break; }
            }
        }
        return true;
    }
};

int load(const char *path, NcFile &f) {
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        set_error("cannot open %s", path);
        return MG_EINVAL;
    }
    fseek(fp, 0, SEEK_END);
    const long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    f.raw.resize(sz > 0 ? (size_t)sz : 0);
    const size_t got = f.raw.empty() ? 0 : fread(f.raw.data(), 1, f.raw.size(), fp);
    fclose(fp);
    if (got != f.raw.size() || !f.parse()) {
        set_error("%s is not a netCDF classic (CDF-1 / CDF-2) file", path);
        return MG_EINVAL;
    }
    return MG_OK;
}

// the element blocks of an ExodusII file: connect1..connectN (ExodusII names)
int blocks(const NcFile &f, int *npe, std::string *etype, int64_t *n_elems) {
    const int nblk = (int)f.dim_len("num_el_blk");
    if (nblk <= 0) {
        set_error("ExodusII file without element blocks");
        return MG_EINVAL;
    }
    *n_elems = 0;
    *npe = 0;
    for (int b = 1; b <= nblk; b++) {
        const std::string cn = "connect" + std::to_string(b);
        auto it = f.vars.find(cn);
        if (it == f.vars.end() || it->second.dims.size() != 2) {
            set_error("ExodusII block %d has no connectivity", b);
            return MG_EINVAL;
        }
        const RVar &cv = it->second;
        // an element block is a fixed-size [num_el_in_blk][num_nod_per_el] integer table
        const uint64_t rows = f.dims[cv.dims[0]].second, cols = f.dims[cv.dims[1]].second;
        if ((int)cv.dims[0] == f.record_dim || (int)cv.dims[1] == f.record_dim || cols < 1 || cols > 64 ||
            rows > f.raw.size() || type_size(cv.type) == 0 || cv.type == kNcChar) {
            set_error("ExodusII block %d: connectivity is not an element x node table", b);
            return MG_EINVAL;
        }
        const int n = (int)cols;
        std::string t;
        auto at = it->second.text_atts.find("elem_type");
        if (at != it->second.text_atts.end()) t = at->second;
        for (char &c : t) c = (char)toupper((unsigned char)c);
        if (b == 1) {
            *npe = n;
            *etype = t;
        } else if (n != *npe) {
            set_error("ExodusII blocks of different element types (%d and %d nodes)", *npe, n);
            return MG_EINVAL;
        }
        *n_elems += (int64_t)rows;
    }
    return MG_OK;
}

}  // namespace
}  // namespace mg

using namespace mg;

static int exodus_write(const char *path, const char *title, int32_t dim, int32_t nodes_per_elem, int64_t n_nodes,
                    const double *coords, int64_t n_elems, const int32_t *conn, int32_t n_nodal_vars,
                    const char *const *nodal_names, const double *nodal_vals, int32_t n_elem_vars,
                    const char *const *elem_names, const double *elem_vals, double time) {
    if (!path || !coords || !conn || (dim != 2 && dim != 3) || n_nodes <= 0 || n_elems <= 0 ||
        (nodes_per_elem != 8 && nodes_per_elem != 4) || n_nodal_vars < 0 || n_elem_vars < 0 ||
        (n_nodal_vars > 0 && (!nodal_names || !nodal_vals)) || (n_elem_vars > 0 && (!elem_names || !elem_vals)) ||
        n_nodes > INT32_MAX || n_elems > INT32_MAX) {
        set_error("mg_exodus_write: invalid argument");
        return MG_EINVAL;
    }
    for (int32_t i = 0; i < n_nodal_vars; i++)
        if (!nodal_names[i]) { set_error("mg_exodus_write: nodal variable %d has no name", i); return MG_EINVAL; }
    for (int32_t i = 0; i < n_elem_vars; i++)
        if (!elem_names[i]) { set_error("mg_exodus_write: element variable %d has no name", i); return MG_EINVAL; }
    // the classic format's 32-bit per-variable size field: every variable below 4 GiB
    if ((uint64_t)std::max<int64_t>(n_nodes, n_elems * nodes_per_elem / 2) * 8 >= 0xFFFFFFFCull) {
        set_error("mg_exodus_write: a variable of %lld values exceeds the classic format's 4 GiB variable size",
                  (long long)std::max<int64_t>(n_nodes, n_elems * nodes_per_elem));
        return MG_EINVAL;
    }
    const int len_name = 33;
    // dimensions
    std::vector<std::pair<std::string, uint32_t>> dims = {
        {"len_string", 33}, {"len_line", 81}, {"four", 4}, {"len_name", (uint32_t)len_name},
        {"time_step", 0}, {"num_dim", (uint32_t)dim}, {"num_nodes", (uint32_t)n_nodes},
        {"num_elem", (uint32_t)n_elems}, {"num_el_blk", 1}, {"num_el_in_blk1", (uint32_t)n_elems},
        {"num_nod_per_el1", (uint32_t)nodes_per_elem}};
    std::map<std::string, int> did;
    auto dim_id = [&](const std::string &n) { return did.at(n); };
    if (n_nodal_vars > 0) dims.push_back({"num_nod_var", (uint32_t)n_nodal_vars});
    if (n_elem_vars > 0) dims.push_back({"num_elem_var", (uint32_t)n_elem_vars});
    for (size_t i = 0; i < dims.size(); i++) did[dims[i].first] = (int)i;
    // variables: fixed-size first, then the record variables
    std::vector<WVar> vars;
    const char *axis[3] = {"coordx", "coordy", "coordz"};
    for (int d = 0; d < dim; d++) {
        std::vector<double> c((size_t)n_nodes);
        for (int64_t i = 0; i < n_nodes; i++) c[i] = coords[i * dim + d];
        vars.push_back(WVar{axis[d], {dim_id("num_nodes")}, {}, kNcDouble, be_doubles(c.data(), n_nodes), false});
    }
    {
        std::vector<std::string> cn = {"X", "Y", "Z"};
        cn.resize(dim);
        vars.push_back(WVar{"coor_names", {dim_id("num_dim"), dim_id("len_name")}, {}, kNcChar,
                            name_table(cn, len_name), false});
    }
    vars.push_back(WVar{"eb_status", {dim_id("num_el_blk")}, {}, kNcInt, be_ints({1}), false});
    vars.push_back(WVar{"eb_prop1", {dim_id("num_el_blk")}, {att_text("name", "ID")}, kNcInt, be_ints({1}), false});
    vars.push_back(WVar{"eb_names", {dim_id("num_el_blk"), dim_id("len_name")}, {}, kNcChar, name_table({""}, len_name),
                        false});
    {
        std::vector<int32_t> c((size_t)n_elems * nodes_per_elem);
        for (size_t i = 0; i < c.size(); i++) {
            if (conn[i] < 0 || conn[i] >= n_nodes) {
                set_error("mg_exodus_write: connectivity entry %zu = %d out of range", i, conn[i]);
                return MG_EINVAL;
            }
            c[i] = conn[i] + 1;  // ExodusII node numbers are 1-based
        }
        const char *et = nodes_per_elem == 8 ? "HEX8" : "QUAD4";
        vars.push_back(WVar{"connect1", {dim_id("num_el_in_blk1"), dim_id("num_nod_per_el1")}, {att_text("elem_type", et)},
                            kNcInt, be_ints(c), false});
    }
    if (n_nodal_vars > 0) {
        std::vector<std::string> nm(nodal_names, nodal_names + n_nodal_vars);
        vars.push_back(WVar{"name_nod_var", {dim_id("num_nod_var"), dim_id("len_name")}, {}, kNcChar,
                            name_table(nm, len_name), false});
    }
    if (n_elem_vars > 0) {
        std::vector<std::string> nm(elem_names, elem_names + n_elem_vars);
        vars.push_back(WVar{"name_elem_var", {dim_id("num_elem_var"), dim_id("len_name")}, {}, kNcChar,
                            name_table(nm, len_name), false});
        vars.push_back(WVar{"elem_var_tab", {dim_id("num_el_blk"), dim_id("num_elem_var")}, {}, kNcInt,
                            be_ints(std::vector<int32_t>((size_t)n_elem_vars, 1)), false});
    }
    vars.push_back(WVar{"time_whole", {dim_id("time_step")}, {}, kNcDouble, be_doubles(&time, 1), true});
    for (int v = 0; v < n_nodal_vars; v++)
        vars.push_back(WVar{"vals_nod_var" + std::to_string(v + 1), {dim_id("time_step"), dim_id("num_nodes")}, {},
                            kNcDouble, be_doubles(nodal_vals + (int64_t)v * n_nodes, n_nodes), true});
    for (int v = 0; v < n_elem_vars; v++)
        vars.push_back(WVar{"vals_elem_var" + std::to_string(v + 1) + "eb1",
                            {dim_id("time_step"), dim_id("num_el_in_blk1")}, {}, kNcDouble,
                            be_doubles(elem_vals + (int64_t)v * n_elems, n_elems), true});
    std::vector<WAtt> gatts = {att_float("api_version", 8.03f), att_float("version", 8.03f),
                               att_int("floating_point_word_size", 8), att_int("file_size", 1),
                               att_int("maximum_name_length", 32),
                               att_text("title", title ? title : "mast-multiphysics_gb300")};
    // header with placeholder offsets, then the offsets once its size is known
    auto header = [&](const std::vector<uint64_t> &begin) {
        Buf h;
        h.b = {'C', 'D', 'F', 2};
        h.u32(1);  // one record (time step)
        h.u32(kTagDim);
        h.u32((uint32_t)dims.size());
        for (auto &d : dims) {
            h.name(d.first);
            h.u32(d.second);
        }
        put_atts(h, gatts);
        h.u32(kTagVar);
        h.u32((uint32_t)vars.size());
        for (size_t i = 0; i < vars.size(); i++) {
            const WVar &v = vars[i];
            h.name(v.name);
            h.u32((uint32_t)v.dims.size());
            for (int d : v.dims) h.u32((uint32_t)d);
            put_atts(h, v.atts);
            h.u32(v.type);
            h.u32((uint32_t)((v.data.size() + 3) & ~(size_t)3));
            h.u64(begin[i]);
        }
        return h;
    };
    std::vector<uint64_t> begin(vars.size(), 0);
    uint64_t off = header(begin).b.size();
    for (size_t i = 0; i < vars.size(); i++)
        if (!vars[i].record) {
            begin[i] = off;
            off += (vars[i].data.size() + 3) & ~(size_t)3;
        }
    for (size_t i = 0; i < vars.size(); i++)
        if (vars[i].record) {
            begin[i] = off;
            off += (vars[i].data.size() + 3) & ~(size_t)3;
        }
    Buf out = header(begin);
    for (int pass = 0; pass < 2; pass++)
        for (const WVar &v : vars)
            if (v.record == (pass == 1)) {
                out.b.insert(out.b.end(), v.data.begin(), v.data.end());
                out.pad4();
            }
    FILE *fp = fopen(path, "wb");
    if (!fp) {
        set_error("cannot write %s", path);
        return MG_EINVAL;
    }
    const size_t put = fwrite(out.b.data(), 1, out.b.size(), fp);
    const int cl = fclose(fp);
    if (put != out.b.size() || cl != 0) {
        set_error("short write to %s", path);
        return MG_EINVAL;
    }
    return MG_OK;
}

static int exodus_read_sizes(const char *path, int32_t *dim, int32_t *nodes_per_elem, int64_t *n_nodes,
                         int64_t *n_elems) {
    if (!path) return MG_EINVAL;
    NcFile f;
    MG_TRY(load(path, f));
    int npe = 0;
    std::string et;
    int64_t ne = 0;
    MG_TRY(blocks(f, &npe, &et, &ne));
    if (dim) *dim = (int32_t)f.dim_len("num_dim");
    if (nodes_per_elem) *nodes_per_elem = npe;
    if (n_nodes) *n_nodes = (int64_t)f.dim_len("num_nodes");
    if (n_elems) *n_elems = ne;
    return MG_OK;
}

static int exodus_read_mesh(const char *path, double *coords, int32_t *conn) {
    if (!path || !coords || !conn) return MG_EINVAL;
    NcFile f;
    MG_TRY(load(path, f));
    const int dim = (int)f.dim_len("num_dim");
    const int64_t nn = (int64_t)f.dim_len("num_nodes");
    int npe = 0;
    std::string et;
    int64_t ne = 0;
    MG_TRY(blocks(f, &npe, &et, &ne));
    if (dim < 1 || dim > 3 || nn <= 0) {
        set_error("ExodusII file without nodes");
        return MG_EINVAL;
    }
    std::vector<double> v;
    if (f.has("coordx")) {
        const char *axis[3] = {"coordx", "coordy", "coordz"};
        for (int d = 0; d < dim; d++) {
            if (!f.values(axis[d], v) || (int64_t)v.size() != nn) {
                set_error("ExodusII coordinate %s missing", axis[d]);
                return MG_EINVAL;
            }
            for (int64_t i = 0; i < nn; i++) coords[i * dim + d] = v[i];
        }
    } else if (f.values("coord", v) && (int64_t)v.size() == dim * nn) {  // [num_dim][num_nodes]
        for (int d = 0; d < dim; d++)
            for (int64_t i = 0; i < nn; i++) coords[i * dim + d] = v[d * nn + i];
    } else {
        set_error("ExodusII file without coordinates");
        return MG_EINVAL;
    }
    int64_t e0 = 0;
    const int nblk = (int)f.dim_len("num_el_blk");
    for (int b = 1; b <= nblk; b++) {
        if (!f.values("connect" + std::to_string(b), v)) {
            set_error("ExodusII block %d connectivity unreadable", b);
            return MG_EINVAL;
        }
        // the table holds exactly the block's elements (blocks() counted them), so the
        // writes stay inside the caller's n_elems x nodes_per_elem array
        if ((int64_t)v.size() % npe != 0 || e0 + (int64_t)v.size() / npe > ne) {
            set_error("ExodusII block %d connectivity has the wrong size", b);
            return MG_EINVAL;
        }
        for (size_t i = 0; i < v.size(); i++) {
            if (!(v[i] >= 1.0 && v[i] <= (double)nn && v[i] == (double)(int64_t)v[i])) {
                set_error("ExodusII block %d: node %g out of range", b, v[i]);
                return MG_EINVAL;
            }
            conn[e0 * npe + (int64_t)i] = (int32_t)((int64_t)v[i] - 1);
        }
        e0 += (int64_t)v.size() / npe;
    }
    return MG_OK;
}

// the ABI entry points: host allocation failures come back as MG_ENOMEM
int mg_exodus_write(const char *path, const char *title, int32_t dim, int32_t nodes_per_elem, int64_t n_nodes,
                    const double *coords, int64_t n_elems, const int32_t *conn, int32_t n_nodal_vars,
                    const char *const *nodal_names, const double *nodal_vals, int32_t n_elem_vars,
                    const char *const *elem_names, const double *elem_vals, double time) {
    try {
        return exodus_write(path, title, dim, nodes_per_elem, n_nodes, coords, n_elems, conn, n_nodal_vars,
                            nodal_names, nodal_vals, n_elem_vars, elem_names, elem_vals, time);
    } catch (const std::bad_alloc &) {
        set_error("mg_exodus_write: out of host memory");
        return MG_ENOMEM;
    }
}

int mg_exodus_read_sizes(const char *path, int32_t *dim, int32_t *nodes_per_elem, int64_t *n_nodes,
                         int64_t *n_elems) {
    try {
        return exodus_read_sizes(path, dim, nodes_per_elem, n_nodes, n_elems);
    } catch (const std::bad_alloc &) {
        set_error("mg_exodus_read_sizes: out of host memory");
        return MG_ENOMEM;
    }
}

int mg_exodus_read_mesh(const char *path, double *coords, int32_t *conn) {
    try {
        return exodus_read_mesh(path, coords, conn);
    } catch (const std::bad_alloc &) {
        set_error("mg_exodus_read_mesh: out of host memory");
        return MG_ENOMEM;
    }
}
