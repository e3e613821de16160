// mesh_io.cu -- reader of CHM's JSON meshes (.mesh + .param) into the C
// ABI's mesh description, host code.
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

int pbsm3d_mesh_read(const char* mesh_path, const char* param_path, pbsm3d_mesh** out) {
    g_mesh_error.clear();
    if (!mesh_path || !out) return PBSM3D_ERR_INVALID_ARG;
    *out = nullptr;
    std::string text, err;
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
    if (geo != M.end() && geo->second.kind == JVal::NUM && geo->second.num == 1) {
        g_mesh_error = "geographic (lat/long) meshes are not supported: project the mesh to metres";
        return PBSM3D_ERR_UNSUPPORTED;
    }
    auto m = std::make_unique<pbsm3d_mesh>();
    const int64_t nv = V->count, nt = E->count;
    auto expect = [&](const char* k, int64_t n) {
        auto f = M.find(k);
        return f == M.end() || f->second.kind != JVal::NUM || (int64_t)f->second.num == n;
    };
    if (!expect("nvertex", nv) || !expect("nelem", nt) || N->count != nt || nt == 0) {
        g_mesh_error = "vertex/elem/neigh counts disagree with nvertex/nelem";
        return PBSM3D_ERR_BAD_MESH;
    }
    m->n_faces = nt;
    m->n_vertices = nv;
    m->vertex = std::move(V->flat);
    m->elem.resize(3 * nt);
    m->neighbor.resize(3 * nt);
    for (int64_t k = 0; k < 3 * nt; ++k) {
        const double e = E->flat[k], n = N->flat[k];
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
        JVal proot;
        if (!read_file(param_path, text, err) || !parse(text, proot, err)) {
            g_mesh_error = err;
            return PBSM3D_ERR_BAD_MESH;
        }
        if (proot.kind != JVal::OBJ) {
            g_mesh_error = "the .param file is not a JSON object";
            return PBSM3D_ERR_BAD_MESH;
        }
        auto column = [&](const char* k, std::vector<double>& dst) -> int {
            auto f = proot.obj.find(k);
            if (f == proot.obj.end()) return 0;
            if (f->second.kind != JVal::NUMARR || f->second.width != 0 || f->second.count != nt) {
                g_mesh_error = std::string("parameter ") + k + " needs one number per face";
                return PBSM3D_ERR_BAD_MESH;
            }
            dst = std::move(f->second.flat);
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
