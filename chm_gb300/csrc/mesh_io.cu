// mesh_io.cu -- reader of CHM's mesh files, JSON (.mesh + .param) or HDF5
// (_mesh.h5 + _param.h5), into the C ABI's mesh description, host code.
//
// The .mesh file is {"mesh": {"vertex": [[x, y, z], ...], "elem": [[v0, v1,
// v2], ...], "neigh": [[f0, f1, f2], ...], "nvertex", "nelem",
// "is_geographic", "proj4", ...}} (triangulation.cpp:206-356); the optional
// .param file maps parameter names to one value per face.  The per-face
// geometry is computed the way CHM's face class does (triangulation.hpp:
// edge(i) = v[cw(i)] - v[ccw(i)] at :1466-1475, the outward unit normal at
// :1443-1463, edge length at :1493-1498, centroid at :1577-1589, and the
// 2-D area unless the "area" parameter gives it, :1830-1856).  The
// neighbour lists are taken as the file gives them, as CHM does.
//
// Parameters carried into the description: area, TPI_mean, TPI_std,
// TPI_neg_frac, TPI_neg_mean, TPI_neg_std, and the vegetation attributes
// CanopyHeight and LAI when the file has them (CHM takes those from the
// landcover table; a .param column of that name stands in here).
// Geographic (lat/long) meshes are refused: the path works in projected
// metres.
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/pbsm3d.h"

namespace {

// A small JSON reader.  Arrays whose elements are all numbers, or all
// number arrays of one width, are kept flattened (1M-face meshes stay a few
// vectors); other arrays are parsed and dropped.
struct JVal {
    enum Kind { NUL, BOOL, NUM, STR, NUMARR, ARR, OBJ } kind = NUL;
    double num = 0;
    std::string str;
    std::vector<double> flat;
    int width = 0;  // NUMARR: 0 = array of numbers, w = array of w-wide number arrays
    int64_t count = 0;
    std::map<std::string, JVal> obj;
};

struct Parser {
    const char* p;
    const char* end;
    std::string err;

    void ws() {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    }
    bool fail(const char* what) {
        if (err.empty()) err = std::string("JSON: ") + what + " at byte " + std::to_string(p - begin);
        return false;
    }
    const char* begin;

    bool number(double& v) {
        // locale-independent; from_chars takes no leading '+'
        auto r = std::from_chars(p < end && *p == '+' ? p + 1 : p, end, v);
        if (r.ec != std::errc()) return fail("bad number");
        p = r.ptr;
        return true;
    }
    bool string(std::string& s) {
        if (*p != '"') return fail("expected string");
        ++p;
        while (p < end && *p != '"') {
            if (*p == '\\') {
                ++p;
                if (p >= end) return fail("bad escape");
                const char c = *p;
                s.push_back(c == 'n' ? '\n' : c == 't' ? '\t' : c);
                if (c == 'u') p += 4;  // \uXXXX: kept as 'u' (names here are ASCII)
                ++p;
            } else {
                s.push_back(*p++);
            }
        }
        if (p >= end) return fail("unterminated string");
        ++p;
        return true;
    }
    bool value(JVal& v, int depth) {
        if (depth > 64) return fail("nesting too deep");
        ws();
        if (p >= end) return fail("unexpected end");
        const char c = *p;
        if (c == '{') {
            v.kind = JVal::OBJ;
            ++p;
            ws();
            if (p < end && *p == '}') {
                ++p;
                return true;
            }
            while (true) {
                ws();
                std::string key;
                if (!string(key)) return false;
                ws();
                if (p >= end || *p != ':') return fail("expected ':'");
                ++p;
                JVal child;
                if (!value(child, depth + 1)) return false;
                v.obj[key] = std::move(child);
                ws();
                if (p < end && *p == ',') {
                    ++p;
                    continue;
                }
                if (p < end && *p == '}') {
                    ++p;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') return array(v, depth);
        if (c == '"') {
            v.kind = JVal::STR;
            return string(v.str);
        }
        if (!strncmp(p, "true", 4)) {
            p += 4;
            v.kind = JVal::BOOL;
            v.num = 1;
            return true;
        }
        if (!strncmp(p, "false", 5)) {
            p += 5;
            v.kind = JVal::BOOL;
            return true;
        }
        if (!strncmp(p, "null", 4)) {
            p += 4;
            v.kind = JVal::NUL;
            return true;
        }
        v.kind = JVal::NUM;
        return number(v.num);
    }
    // an array: flattened when it holds numbers or equal-width number arrays
    bool array(JVal& v, int depth) {
        ++p;  // '['
        v.kind = JVal::NUMARR;
        v.width = -1;
        ws();
        if (p < end && *p == ']') {
            ++p;
            v.width = 0;
            return true;
        }
        bool numeric = true;
        while (true) {
            ws();
            if (p >= end) return fail("unterminated array");
            if (*p == '[' && numeric) {
                // a nested array: numbers only, its width fixed by the first one
                ++p;
                int w = 0;
                ws();
                while (p < end && *p != ']') {
                    double x;
                    ws();
                    if (!number(x)) {
                        numeric = false;
                        return fail("non-numeric nested array");
                    }
                    v.flat.push_back(x);
                    ++w;
                    ws();
                    if (p < end && *p == ',') ++p;
                }
                if (p >= end) return fail("unterminated array");
                ++p;
                if (v.width == -1) v.width = w;
                if (w != v.width) return fail("ragged nested array");
            } else if (numeric && (*p == '-' || *p == '+' || (*p >= '0' && *p <= '9'))) {
                double x;
                if (!number(x)) return false;
                if (v.width == -1) v.width = 0;
                if (v.width != 0) return fail("mixed array");
                v.flat.push_back(x);
            } else {
                // anything else: parse and drop
                numeric = false;
                v.kind = JVal::ARR;
                v.flat.clear();
                JVal tmp;
                if (!value(tmp, depth + 1)) return false;
            }
            ++v.count;
            ws();
            if (p < end && *p == ',') {
                ++p;
                continue;
            }
            if (p < end && *p == ']') {
                ++p;
                if (v.width < 0) v.width = 0;
                return true;
            }
            return fail("expected ',' or ']'");
        }
    }
};

bool read_file(const char* path, std::string& out, std::string& err) {
    FILE* f = fopen(path, "rb");
    if (!f) {
        err = std::string("cannot open ") + path;
        return false;
    }
    fseek(f, 0, SEEK_END);
    const long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    out.resize(n > 0 ? (size_t)n : 0);
    const size_t got = n > 0 ? fread(&out[0], 1, (size_t)n, f) : 0;
    fclose(f);
    if ((long)got != n) {
        err = std::string("short read of ") + path;
        return false;
    }
    return true;
}

bool parse(const std::string& text, JVal& root, std::string& err) {
    Parser ps{text.data(), text.data() + text.size(), {}, text.data()};
    if (!ps.value(root, 0)) {
        err = ps.err;
        return false;
    }
    return true;
}

// ---------------------------------------------------------------- HDF5
// A reader of the part of the HDF5 file format that CHM's mesh and parameter
// files use (written by CHM's triangulation::to_hdf5 and its partition
// tools; read by triangulation::load_mesh_from_h5 and load_hdf5_parameters,
// triangulation.cpp:724-1035, 1237-1383), restated from the published HDF5
// file-format specification: superblock versions 0 and 1; groups held in
// symbol tables (version-1 B-trees of type 0, symbol-table nodes, local
// heaps); version-1 object headers with continuation blocks; datasets with
// contiguous or compact layout (layout message versions 1-3); fixed-point,
// floating-point (IEEE, either byte order), fixed-length string and array
// datatypes; attributes of message version 1-3.  Chunked or filtered datasets, the
// global heap (variable-length strings) and superblock version 2+ are
// refused with a message.  Every offset is checked against the file size.
struct H5 {
    std::vector<unsigned char> d;
    int so = 8, sl = 8;  // sizes of offsets and lengths
    std::string err;

    bool has(uint64_t p, uint64_t n) const { return p <= d.size() && n <= d.size() - p; }
    uint64_t uint(uint64_t p, int n) const {
        uint64_t v = 0;
        for (int k = n - 1; k >= 0; --k) v = (v << 8) | d[p + k];
        return v;
    }
    uint64_t uint_be(uint64_t p, int n) const {
        uint64_t v = 0;
        for (int k = 0; k < n; ++k) v = (v << 8) | d[p + k];
        return v;
    }
    uint64_t off(uint64_t p) const { return uint(p, so); }
    uint64_t len(uint64_t p) const { return uint(p, sl); }
    bool fail(const std::string& m) {
        if (err.empty()) err = m;
        return false;
    }
};

struct H5Msg {
    int type;
    uint64_t pos, size;  // body position and size in the file
};

struct H5Type {
    int cls = -1, size = 0, count = 1;  // count > 1: an array of count base elements
    int base_cls = -1, base_size = 0;
    bool is_signed = false;
    bool big = false;  // big-endian elements
};

bool h5_open(H5& f, const char* path) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return f.fail(std::string("cannot open ") + path);
    std::fseek(fp, 0, SEEK_END);
    const long n = std::ftell(fp);
    std::fseek(fp, 0, SEEK_SET);
    f.d.resize(n > 0 ? (size_t)n : 0);
    const size_t got = f.d.empty() ? 0 : std::fread(f.d.data(), 1, f.d.size(), fp);
    std::fclose(fp);
    if (got != f.d.size()) return f.fail(std::string("cannot read ") + path);
    return true;
}

bool is_hdf5(const char* path) {
    FILE* fp = std::fopen(path, "rb");
    if (!fp) return false;
    unsigned char sig[8] = {0};
    const size_t n = std::fread(sig, 1, 8, fp);
    std::fclose(fp);
    static const unsigned char kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    return n == 8 && std::memcmp(sig, kSig, 8) == 0;
}

// The root group's symbol-table entry: its B-tree and local heap.
bool h5_root(H5& f, uint64_t& btree, uint64_t& heap) {
    if (!f.has(0, 24)) return f.fail("truncated HDF5 superblock");
    const int ver = f.d[8];
    if (ver > 1) return f.fail("HDF5 superblock version " + std::to_string(ver) + " is not supported");
    f.so = f.d[13];
    f.sl = f.d[14];
    if ((f.so != 4 && f.so != 8) || (f.sl != 4 && f.sl != 8)) return f.fail("unsupported HDF5 offset/length sizes");
    uint64_t p = ver == 0 ? 24 : 28;
    p += 4 * (uint64_t)f.so;  // base, free-space, end-of-file and driver addresses
    if (!f.has(p, 2 * f.so + 24)) return f.fail("truncated HDF5 root symbol-table entry");
    if (f.uint(p + 2 * f.so, 4) != 1) return f.fail("the HDF5 root group has no cached symbol table");
    btree = f.off(p + 2 * f.so + 8);
    heap = f.off(p + 3 * f.so + 8);
    return true;
}

bool h5_heap_data(H5& f, uint64_t heap, uint64_t& data, uint64_t& size) {
    if (!f.has(heap, 8 + 2 * f.sl + f.so) || std::memcmp(&f.d[heap], "HEAP", 4) != 0)
        return f.fail("bad HDF5 local heap");
    size = f.len(heap + 8);
    data = f.off(heap + 8 + 2 * f.sl);
    if (!f.has(data, size)) return f.fail("HDF5 local heap out of the file");
    return true;
}

// Members of a group: name -> (object header address, cached B-tree, heap).
struct H5Entry {
    uint64_t ohdr = 0, btree = 0, heap = 0;
    bool cached_group = false;
};
bool h5_members(H5& f, uint64_t btree, uint64_t heap, std::map<std::string, H5Entry>& out, int depth = 0) {
    uint64_t hd, hs;
    if (depth > 32) return f.fail("HDF5 group B-tree too deep");
    if (!h5_heap_data(f, heap, hd, hs)) return false;
    if (!f.has(btree, 8 + 2 * f.so) || std::memcmp(&f.d[btree], "TREE", 4) != 0 || f.d[btree + 4] != 0)
        return f.fail("bad HDF5 group B-tree node");
    const int level = f.d[btree + 5];
    const int n = (int)f.uint(btree + 6, 2);
    uint64_t q = btree + 8 + 2 * f.so;
    for (int i = 0; i < n; ++i) {
        q += f.sl;  // key
        if (!f.has(q, f.so)) return f.fail("truncated HDF5 B-tree node");
        const uint64_t child = f.off(q);
        q += f.so;
        if (level > 0) {
            if (!h5_members(f, child, heap, out, depth + 1)) return false;
            continue;
        }
        if (!f.has(child, 8) || std::memcmp(&f.d[child], "SNOD", 4) != 0) return f.fail("bad HDF5 symbol-table node");
        const int ns = (int)f.uint(child + 6, 2);
        uint64_t e = child + 8;
        const uint64_t esz = 2 * (uint64_t)f.so + 24;
        for (int k = 0; k < ns; ++k, e += esz) {
            if (!f.has(e, esz)) return f.fail("truncated HDF5 symbol-table node");
            const uint64_t name = f.off(e);
            if (name >= hs) return f.fail("HDF5 link name out of its heap");
            const char* c = reinterpret_cast<const char*>(&f.d[hd + name]);
            const size_t L = strnlen(c, hs - name);
            H5Entry en;
            en.ohdr = f.off(e + f.so);
            if (f.uint(e + 2 * f.so, 4) == 1) {
                en.cached_group = true;
                en.btree = f.off(e + 2 * f.so + 8);
                en.heap = f.off(e + 3 * f.so + 8);
            }
            out[std::string(c, L)] = en;
        }
    }
    return true;
}

// The messages of a version-1 object header (continuations followed).
bool h5_messages(H5& f, uint64_t addr, std::vector<H5Msg>& msgs) {
    if (!f.has(addr, 16) || f.d[addr] != 1) return f.fail("unsupported HDF5 object header (version 1 expected)");
    const int nm = (int)f.uint(addr + 2, 2);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, f.uint(addr + 8, 4)}};
    for (size_t b = 0; b < blocks.size() && (int)msgs.size() < nm; ++b) {
        if (b > 64) return f.fail("too many HDF5 header continuations");
        const uint64_t start = blocks[b].first, end = start + blocks[b].second;
        if (!f.has(start, blocks[b].second)) return f.fail("HDF5 object header out of the file");
        for (uint64_t q = start; q + 8 <= end && (int)msgs.size() < nm;) {
            const int type = (int)f.uint(q, 2);
            const uint64_t size = f.uint(q + 2, 2);
            if (q + 8 + size > end) return f.fail("HDF5 header message overruns its block");
            if (type == 0x10) {
                if (size < (uint64_t)(f.so + f.sl)) return f.fail("bad HDF5 continuation message");
                blocks.push_back({f.off(q + 8), f.len(q + 8 + f.so)});
            }
            msgs.push_back(H5Msg{type, q + 8, size});
            q += 8 + size;
        }
    }
    return true;
}

bool h5_type(H5& f, uint64_t p, uint64_t n, H5Type& t) {
    if (n < 8 || !f.has(p, n)) return f.fail("truncated HDF5 datatype");
    const int cls = f.d[p] & 15, ver = f.d[p] >> 4;
    const unsigned bits = (unsigned)f.uint(p + 1, 3);
    t.cls = cls;
    t.size = (int)f.uint(p + 4, 4);
    if (cls == 0 || cls == 1) {
        if (cls == 1 && (bits & 0x40)) return f.fail("VAX-order HDF5 floats are not supported");
        t.big = bits & 1;
        t.is_signed = cls == 0 && (bits & 8);
        t.base_cls = cls;
        t.base_size = t.size;
        if ((cls == 1 && t.size != 4 && t.size != 8) || (cls == 0 && (t.size < 1 || t.size > 8)))
            return f.fail("unsupported HDF5 number size " + std::to_string(t.size));
        return true;
    }
    if (cls == 3) return true;  // fixed-length string
    if (cls == 10) {            // array: rank, dims, then the base type
        if (ver < 2 || n < 12) return f.fail("unsupported HDF5 array datatype");
        const int rank = f.d[p + 8];
        uint64_t q = p + 8 + (ver == 2 ? 4 : 1);  // rank (+ 3 reserved bytes in version 2)
        int64_t count = 1;
        for (int k = 0; k < rank; ++k, q += 4) {
            if (!f.has(q, 4)) return f.fail("truncated HDF5 array datatype");
            count *= (int64_t)f.uint(q, 4);
            if (count <= 0 || count > (1 << 20)) return f.fail("unsupported HDF5 array size");
        }
        if (ver == 2) q += 4 * (uint64_t)rank;  // permutation indices
        H5Type b;
        if (q > p + n || !h5_type(f, q, p + n - q, b) || (b.cls != 0 && b.cls != 1)) {
            return f.fail("unsupported HDF5 array base type");
        }
        t.count = (int)count;
        t.base_cls = b.cls;
        t.base_size = b.size;
        t.is_signed = b.is_signed;
        t.big = b.big;
        return true;
    }
    return f.fail("unsupported HDF5 datatype class " + std::to_string(cls));
}

double h5_value(const H5& f, uint64_t p, const H5Type& t) {
    auto raw = [&](int n) { return t.big ? f.uint_be(p, n) : f.uint(p, n); };
    if (t.base_cls == 1) {
        if (t.base_size == 8) {
            double v;
            const uint64_t u = raw(8);
            std::memcpy(&v, &u, 8);
            return v;
        }
        float v;
        const uint32_t u = (uint32_t)raw(4);
        std::memcpy(&v, &u, 4);
        return v;
    }
    const uint64_t u = raw(t.base_size);
    if (t.is_signed && t.base_size < 8 && (u >> (8 * t.base_size - 1)) & 1)
        return (double)(int64_t)(u | (~uint64_t(0) << (8 * t.base_size)));
    return t.is_signed ? (double)(int64_t)u : (double)u;
}

// A numeric dataset (scalar elements or arrays of them), as doubles: n rows
// of `width` values.
bool h5_dataset(H5& f, uint64_t ohdr, std::vector<double>& out, int64_t& n, int& width) {
    std::vector<H5Msg> msgs;
    if (!h5_messages(f, ohdr, msgs)) return false;
    H5Type t;
    bool have_t = false, have_space = false, have_layout = false;
    uint64_t data = 0, bytes = 0;
    n = 0;
    for (const H5Msg& m : msgs) {
        const uint64_t p = m.pos;
        if (m.type == 0x0001) {  // dataspace
            if (m.size < 8) return f.fail("bad HDF5 dataspace");
            const int ver = f.d[p], rank = f.d[p + 1];
            const uint64_t q = p + (ver == 1 ? 8 : 4);
            if (rank != 1) return f.fail("HDF5 mesh datasets are one-dimensional");
            if (!f.has(q, f.sl)) return f.fail("truncated HDF5 dataspace");
            n = (int64_t)f.len(q);
            have_space = true;
        } else if (m.type == 0x0003) {
            if (!h5_type(f, p, m.size, t)) return false;
            have_t = true;
        } else if (m.type == 0x000B) {
            return f.fail("filtered (compressed) HDF5 datasets are not supported");
        } else if (m.type == 0x0008) {  // data layout
            const int ver = f.d[p];
            if (ver == 3) {
                const int cls = f.d[p + 1];
                if (cls == 1) {
                    data = f.off(p + 2);
                    bytes = f.len(p + 2 + f.so);
                } else if (cls == 0) {
                    bytes = f.uint(p + 2, 2);
                    data = p + 4;
                } else {
                    return f.fail("chunked HDF5 datasets are not supported");
                }
            } else if (ver == 1 || ver == 2) {
                const int rank = f.d[p + 1], cls = f.d[p + 2];
                if (cls == 1) {
                    data = f.off(p + 8);
                    bytes = UINT64_MAX;  // from the dataspace and the type
                } else if (cls == 0) {
                    const uint64_t q = p + 8 + 4 * (uint64_t)rank;
                    bytes = f.uint(q, 4);
                    data = q + 4;
                } else {
                    return f.fail("chunked HDF5 datasets are not supported");
                }
            } else {
                return f.fail("unsupported HDF5 layout message version " + std::to_string(ver));
            }
            have_layout = true;
        }
    }
    if (!have_t || !have_space || !have_layout) return f.fail("HDF5 dataset lacks its type, space or layout");
    if (t.cls == 3) return f.fail("string HDF5 dataset where numbers were expected");
    if (n < 0 || (uint64_t)n > f.d.size() || t.count < 1 || t.base_size < 1)
        return f.fail("HDF5 dataset larger than its file");
    const uint64_t need = (uint64_t)n * t.count * t.base_size;
    if (bytes != UINT64_MAX && bytes < need) return f.fail("HDF5 dataset shorter than its dataspace");
    if (!f.has(data, need)) return f.fail("HDF5 dataset data out of the file");
    width = t.count;
    out.resize((size_t)n * t.count);
    for (uint64_t k = 0; k < (uint64_t)n * t.count; ++k) out[k] = h5_value(f, data + k * t.base_size, t);
    return true;
}

// Attribute `name` of an object: a fixed-length string, or a number.
bool h5_attribute(H5& f, uint64_t ohdr, const std::string& name, std::string* str, double* num, bool& found) {
    found = false;
    std::vector<H5Msg> msgs;
    if (!h5_messages(f, ohdr, msgs)) return false;
    for (const H5Msg& m : msgs) {
        if (m.type != 0x000C || m.size < 8) continue;
        const uint64_t p = m.pos;
        const int ver = f.d[p];
        const uint64_t ns = f.uint(p + 2, 2), dts = f.uint(p + 4, 2), dss = f.uint(p + 6, 2);
        auto pad = [&](uint64_t x) { return ver == 1 ? (x + 7) / 8 * 8 : x; };
        uint64_t q = p + (ver == 3 ? 9 : 8);
        if (q + pad(ns) + pad(dts) + pad(dss) > p + m.size) return f.fail("bad HDF5 attribute message");
        const char* c = reinterpret_cast<const char*>(&f.d[q]);
        if (std::string(c, strnlen(c, ns)) != name) continue;
        q += pad(ns);
        H5Type t;
        if (!h5_type(f, q, dts, t)) return false;
        q += pad(dts) + pad(dss);
        if (!f.has(q, (uint64_t)t.size)) return f.fail("HDF5 attribute data out of the file");
        found = true;
        if (t.cls == 3) {
            const char* v = reinterpret_cast<const char*>(&f.d[q]);
            if (str) *str = std::string(v, strnlen(v, (size_t)t.size));
        } else if (t.cls == 0 || t.cls == 1) {
            if (num) *num = h5_value(f, q, t);
        } else {
            return f.fail("unsupported HDF5 attribute type for " + name);
        }
        return true;
    }
    return true;
}

// CHM's HDF5 mesh: /mesh/vertex [n][3] f64, /mesh/elem and /mesh/neighbor
// [n][3] int, /mesh/cell_global_id, attributes "/mesh/version", "/mesh/proj4",
// "/mesh/is_geographic", "/mesh/is_partition" on the root group.
bool read_h5_mesh(const char* path, std::vector<double>& vertex, std::vector<double>& elem,
                  std::vector<double>& neigh, int64_t& nv, int64_t& nt, bool& geographic, std::string& err) {
    H5 f;
    uint64_t bt, hp;
    std::map<std::string, H5Entry> root, mesh;
    auto bad = [&]() {
        err = f.err.empty() ? "bad HDF5 mesh" : f.err;
        return false;
    };
    if (!h5_open(f, path) || !h5_root(f, bt, hp) || !h5_members(f, bt, hp, root)) return bad();
    // the root group's own object header: its symbol-table entry is the superblock's
    const uint64_t root_ohdr = f.off((f.d[8] == 0 ? 24 : 28) + 4 * (uint64_t)f.so + f.so);
    auto it = root.find("mesh");
    if (it == root.end() || !it->second.cached_group) {
        err = "no /mesh group";
        return false;
    }
    if (!h5_members(f, it->second.btree, it->second.heap, mesh)) return bad();
    double part = 0, geo = 0;
    bool found;
    if (!h5_attribute(f, root_ohdr, "/mesh/is_partition", nullptr, &part, found)) return bad();
    if (found && part != 0) {
        err = "partitioned HDF5 meshes (one file of a multi-process partition) are not supported: load the "
              "unpartitioned mesh";
        return false;
    }
    if (!h5_attribute(f, root_ohdr, "/mesh/is_geographic", nullptr, &geo, found)) return bad();
    geographic = found && geo != 0;
    auto dataset = [&](const char* k, std::vector<double>& out, int64_t& n, int w) {
        auto e = mesh.find(k);
        int width = 0;
        if (e == mesh.end()) return f.fail(std::string("no /mesh/") + k + " dataset");
        if (!h5_dataset(f, e->second.ohdr, out, n, width)) return false;
        if (width != w) return f.fail(std::string("/mesh/") + k + " must have " + std::to_string(w) + " values a row");
        return true;
    };
    int64_t ne = 0;
    if (!dataset("vertex", vertex, nv, 3) || !dataset("elem", elem, nt, 3) || !dataset("neighbor", neigh, ne, 3))
        return bad();
    if (ne != nt) {
        err = "/mesh/neighbor and /mesh/elem have different lengths";
        return false;
    }
    std::vector<double> gid;
    int64_t ng = 0;
    if (mesh.count("cell_global_id")) {
        if (!dataset("cell_global_id", gid, ng, 1)) return bad();
        for (int64_t i = 0; i < ng; ++i)
            if (gid[i] != (double)i) {
                err = "cell_global_id is not the file order (a partitioned mesh)";
                return false;
            }
    }
    return true;
}

// CHM's HDF5 parameter file: one f64 dataset of n values per parameter in
// the /parameters group.
bool read_h5_params(const char* path, int64_t nt, std::map<std::string, std::vector<double>>& cols,
                    std::string& err) {
    H5 f;
    uint64_t bt, hp;
    std::map<std::string, H5Entry> root, pars;
    if (!h5_open(f, path) || !h5_root(f, bt, hp) || !h5_members(f, bt, hp, root)) {
        err = f.err;
        return false;
    }
    auto it = root.find("parameters");
    if (it == root.end() || !it->second.cached_group) {
        err = "no /parameters group";
        return false;
    }
    if (!h5_members(f, it->second.btree, it->second.heap, pars)) {
        err = f.err;
        return false;
    }
    for (auto& kv : pars) {
        std::vector<double> v;
        int64_t n = 0;
        int width = 0;
        if (!h5_dataset(f, kv.second.ohdr, v, n, width)) {
            err = "parameter " + kv.first + ": " + f.err;
            return false;
        }
        if (width != 1 || n != nt) {
            err = "parameter " + kv.first + " needs one number per face";
            return false;
        }
        cols[kv.first] = std::move(v);
    }
    return true;
}

}  // namespace

struct pbsm3d_mesh {
    int64_t n_faces = 0, n_vertices = 0;
    std::vector<double> vertex;  // [3 nv]
    std::vector<int32_t> elem, neighbor;
    std::vector<double> edge_length, edge_normal, area, center;
    std::vector<double> canopy, lai, tpi[5];
};

static thread_local std::string g_mesh_error;

extern "C" {

const char* pbsm3d_mesh_last_error(void) { return g_mesh_error.c_str(); }

static int mesh_read(const char* mesh_path, const char* param_path, pbsm3d_mesh** out);

int pbsm3d_mesh_read(const char* mesh_path, const char* param_path, pbsm3d_mesh** out) {
    // no C++ exception (an allocation failing on a corrupt file) crosses the C ABI
    try {
        return mesh_read(mesh_path, param_path, out);
    } catch (const std::exception& e) {
        g_mesh_error = std::string("mesh reader: ") + e.what();
        return PBSM3D_ERR_BAD_MESH;
    }
}

static int mesh_read(const char* mesh_path, const char* param_path, pbsm3d_mesh** out) {
    g_mesh_error.clear();
    if (!mesh_path || !out) return PBSM3D_ERR_INVALID_ARG;
    *out = nullptr;
    std::string text, err;
    std::vector<double> vflat, eflat, nflat;
    int64_t nv = 0, nt = 0;
    bool geographic = false;
    if (is_hdf5(mesh_path)) {
        if (!read_h5_mesh(mesh_path, vflat, eflat, nflat, nv, nt, geographic, err)) {
            g_mesh_error = err;
            return PBSM3D_ERR_BAD_MESH;
        }
        if (nt == 0) {
            g_mesh_error = "the mesh has no faces";
            return PBSM3D_ERR_BAD_MESH;
        }
    } else {
        JVal root;
        if (!read_file(mesh_path, text, err) || !parse(text, root, err)) {
            g_mesh_error = err;
            return PBSM3D_ERR_BAD_MESH;
        }
        text.clear();
        text.shrink_to_fit();
        auto it = root.obj.find("mesh");
        if (root.kind != JVal::OBJ || it == root.obj.end() || it->second.kind != JVal::OBJ) {
            g_mesh_error = "no \"mesh\" object";
            return PBSM3D_ERR_BAD_MESH;
        }
        auto& M = it->second.obj;
        auto need = [&](const char* k, int width) -> JVal* {
            auto f = M.find(k);
            if (f == M.end() || f->second.kind != JVal::NUMARR || f->second.width != width) return nullptr;
            return &f->second;
        };
        JVal *V = need("vertex", 3), *E = need("elem", 3), *N = need("neigh", 3);
        if (!V || !E || !N) {
            g_mesh_error = "mesh.vertex, mesh.elem and mesh.neigh must be arrays of 3-element arrays";
            return PBSM3D_ERR_BAD_MESH;
        }
        auto geo = M.find("is_geographic");
        geographic = geo != M.end() && geo->second.kind == JVal::NUM && geo->second.num == 1;
        nv = V->count;
        nt = E->count;
        auto expect = [&](const char* k, int64_t n) {
            auto f = M.find(k);
            return f == M.end() || f->second.kind != JVal::NUM || (int64_t)f->second.num == n;
        };
        if (!expect("nvertex", nv) || !expect("nelem", nt) || N->count != nt || nt == 0) {
            g_mesh_error = "vertex/elem/neigh counts disagree with nvertex/nelem";
            return PBSM3D_ERR_BAD_MESH;
        }
        vflat = std::move(V->flat);
        eflat = std::move(E->flat);
        nflat = std::move(N->flat);
    }
    if (geographic) {
        g_mesh_error = "geographic (lat/long) meshes are not supported: project the mesh to metres";
        return PBSM3D_ERR_UNSUPPORTED;
    }
    auto m = std::make_unique<pbsm3d_mesh>();
    m->n_faces = nt;
    m->n_vertices = nv;
    m->vertex = std::move(vflat);
    m->elem.resize(3 * nt);
    m->neighbor.resize(3 * nt);
    for (int64_t k = 0; k < 3 * nt; ++k) {
        const double e = eflat[k], n = nflat[k];
        if (!(e >= 0 && e < nv) || e != std::floor(e) || !(n >= -1 && n < nt) || n != std::floor(n)) {
            g_mesh_error = "elem or neigh index out of range at face " + std::to_string(k / 3);
            return PBSM3D_ERR_BAD_MESH;
        }
        m->elem[k] = (int32_t)e;
        m->neighbor[k] = (int32_t)n;
    }
    // per-face geometry, CHM's operation order
    m->edge_length.resize(3 * nt);
    m->edge_normal.resize(6 * nt);
    m->area.resize(nt);
    m->center.resize(3 * nt);
    for (int64_t f = 0; f < nt; ++f) {
        const double* p[3];
        for (int k = 0; k < 3; ++k) p[k] = &m->vertex[3 * (int64_t)m->elem[3 * f + k]];
        double ex[3], ey[3];
        for (int i = 0; i < 3; ++i) {
            const double* a = p[(i + 1) % 3];
            const double* b = p[(i + 2) % 3];
            ex[i] = b[0] - a[0];
            ey[i] = b[1] - a[1];
        }
        for (int i = 0; i < 3; ++i) {
            double nx = ey[i], ny = -ex[i];
            const int i1 = (i + 1) % 3;
            const double D = ex[i1] * nx + ey[i1] * ny;
            if (D > 0) {
                nx = -nx;
                ny = -ny;
            }
            const double len = std::sqrt(nx * nx + ny * ny);
            m->edge_normal[6 * f + 2 * i] = nx / len;
            m->edge_normal[6 * f + 2 * i + 1] = ny / len;
            m->edge_length[3 * f + i] = std::sqrt(ex[i] * ex[i] + ey[i] * ey[i]);
        }
        m->area[f] = ((p[1][0] - p[0][0]) * (p[2][1] - p[0][1]) - (p[1][1] - p[0][1]) * (p[2][0] - p[0][0])) / 2.0;
        for (int c = 0; c < 3; ++c) m->center[3 * f + c] = (p[0][c] + p[1][c] + p[2][c]) / 3.0;
    }
    if (param_path && *param_path) {
        // one value per face for each parameter, from CHM's JSON .param or
        // its HDF5 parameter file
        std::map<std::string, std::vector<double>> cols;
        if (is_hdf5(param_path)) {
            if (!read_h5_params(param_path, nt, cols, err)) {
                g_mesh_error = err;
                return PBSM3D_ERR_BAD_MESH;
            }
        } else {
            JVal proot;
            if (!read_file(param_path, text, err) || !parse(text, proot, err)) {
                g_mesh_error = err;
                return PBSM3D_ERR_BAD_MESH;
            }
            if (proot.kind != JVal::OBJ) {
                g_mesh_error = "the .param file is not a JSON object";
                return PBSM3D_ERR_BAD_MESH;
            }
            static const char* kUsed[] = {"area",         "TPI_mean",     "TPI_std",      "TPI_neg_frac",
                                          "TPI_neg_mean", "TPI_neg_std",  "CanopyHeight", "LAI"};
            for (auto& kv : proot.obj) {
                if (kv.second.kind != JVal::NUMARR || kv.second.width != 0) {
                    for (const char* u : kUsed)
                        if (kv.first == u) {
                            g_mesh_error = "parameter " + kv.first + " needs one number per face";
                            return PBSM3D_ERR_BAD_MESH;
                        }
                    continue;
                }
                cols[kv.first] = std::move(kv.second.flat);
            }
        }
        auto column = [&](const char* k, std::vector<double>& dst) -> int {
            auto f = cols.find(k);
            if (f == cols.end()) return 0;
            if ((int64_t)f->second.size() != nt) {
                g_mesh_error = std::string("parameter ") + k + " needs one number per face";
                return PBSM3D_ERR_BAD_MESH;
            }
            dst = std::move(f->second);
            return 0;
        };
        std::vector<double> a;
        int rc = column("area", a);
        if (!rc && !a.empty()) m->area = std::move(a);
        const char* tp[5] = {"TPI_mean", "TPI_std", "TPI_neg_frac", "TPI_neg_mean", "TPI_neg_std"};
        for (int k = 0; k < 5 && !rc; ++k) rc = column(tp[k], m->tpi[k]);
        if (!rc) rc = column("CanopyHeight", m->canopy);
        if (!rc) rc = column("LAI", m->lai);
        if (rc) return rc;
    }
    *out = m.release();
    return 0;
}

int pbsm3d_mesh_describe(const pbsm3d_mesh* m, pbsm3d_mesh_desc* d) {
    if (!m || !d) return PBSM3D_ERR_INVALID_ARG;
    *d = pbsm3d_mesh_desc{};
    d->n_faces = m->n_faces;
    d->neighbor = m->neighbor.data();
    d->edge_length = m->edge_length.data();
    d->edge_normal = m->edge_normal.data();
    d->area = m->area.data();
    d->center = m->center.data();
    d->canopy_height = m->canopy.empty() ? nullptr : m->canopy.data();
    d->lai = m->lai.empty() ? nullptr : m->lai.data();
    const double** tp[5] = {&d->tpi_mean, &d->tpi_std, &d->tpi_neg_frac, &d->tpi_neg_mean, &d->tpi_neg_std};
    for (int k = 0; k < 5; ++k) *tp[k] = m->tpi[k].empty() ? nullptr : m->tpi[k].data();
    return 0;
}

int pbsm3d_mesh_arrays(const pbsm3d_mesh* m, int64_t* n_vertices, const double** vertex, const int32_t** elem) {
    if (!m) return PBSM3D_ERR_INVALID_ARG;
    if (n_vertices) *n_vertices = m->n_vertices;
    if (vertex) *vertex = m->vertex.data();
    if (elem) *elem = m->elem.data();
    return 0;
}

void pbsm3d_mesh_free(pbsm3d_mesh* m) { delete m; }

}  // extern "C"
