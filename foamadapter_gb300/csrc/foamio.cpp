// OpenFOAM files on the host: the ASCII polyMesh a case is read from and the
// volScalarField files results are written to.  In FoamAdapter these are the
// steps before and after the hot path: MeshAdapter builds the NeoN mesh from
// Foam::fvMesh (src/datastructures/meshAdapter.cpp:59-136) and writers.cpp
// writes NeoN fields back as OpenFOAM fields.  Geometry is computed by
// fvgb_geometry_compute (meshgen.cpp), the same routine the box builder uses.
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "fvgb.h"
#include "fvgb_host_common.h"

#define FVGB_CHECK_ARG(cond, msg) \
    do {                          \
        if (!(cond)) return fvgb_fail(FVGB_ERR_INVALID_ARG, msg); \
    } while (0)

namespace {

// Tokens of an OpenFOAM dictionary/list file: words (numbers, names,
// List<scalar>) and the punctuation ( ) { } ; -- comments removed.
struct Lexer {
    std::string s;
    size_t i = 0;
    bool punct(char c) const { return c == '(' || c == ')' || c == '{' || c == '}' || c == ';'; }
    void skip() {
        for (;;) {
            while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
            if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '/') {
                while (i < s.size() && s[i] != '\n') ++i;
            } else if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '*') {
                const size_t e = s.find("*/", i + 2);
                i = e == std::string::npos ? s.size() : e + 2;
            } else {
                return;
            }
        }
    }
    bool next(std::string& t) {
        skip();
        if (i >= s.size()) return false;
        if (punct(s[i])) {
            t.assign(1, s[i++]);
            return true;
        }
        if (s[i] == '"') {  // quoted string
            const size_t e = s.find('"', i + 1);
            const size_t end = e == std::string::npos ? s.size() : e + 1;
            t = s.substr(i, end - i);
            i = end;
            return true;
        }
        const size_t b = i;
        while (i < s.size() && !std::isspace((unsigned char)s[i]) && !punct(s[i])) ++i;
        t = s.substr(b, i - b);
        return true;
    }
    bool expect(const char* want) {
        std::string t;
        return next(t) && t == want;
    }
};

bool read_text(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

// Skips the FoamFile header (if any); false when it declares a binary file.
bool skip_header(Lexer& lx) {
    const size_t save = lx.i;
    std::string t;
    if (!lx.next(t) || t != "FoamFile") {
        lx.i = save;
        return true;
    }
    if (!lx.expect("{")) return false;
    int depth = 1;
    std::string prev;
    while (depth > 0 && lx.next(t)) {
        if (t == "{") ++depth;
        else if (t == "}") --depth;
        else if (prev == "format" && t == "binary") return false;
        prev = t;
    }
    return depth == 0;
}

bool to_long(const std::string& t, long& v) {
    char* e = nullptr;
    v = std::strtol(t.c_str(), &e, 10);
    return e && *e == '\0' && !t.empty();
}

bool to_double(const std::string& t, double& v) {
    char* e = nullptr;
    v = std::strtod(t.c_str(), &e);
    return e && *e == '\0' && !t.empty();
}

// "N ( ... )": the count and the opening parenthesis
bool list_start(Lexer& lx, long& n) {
    std::string t;
    return lx.next(t) && to_long(t, n) && n >= 0 && lx.expect("(");
}

bool read_labels(const std::string& path, std::vector<int32_t>& out, bool& binary) {
    std::string text;
    if (!read_text(path, text)) return false;
    Lexer lx{text};
    binary = !skip_header(lx);
    if (binary) return false;
    long n;
    if (!list_start(lx, n)) return false;
    out.resize((size_t)n);
    std::string t;
    for (long k = 0; k < n; ++k) {
        long v;
        if (!lx.next(t) || !to_long(t, v)) return false;
        out[(size_t)k] = (int32_t)v;
    }
    return lx.expect(")");
}

struct Patch {
    std::string name, type;
    long n_faces = 0, start = 0;
};

}  // namespace

struct fvgb_polymesh {
    std::vector<double> points;
    std::vector<Patch> patches;  // every patch, in file order
    std::vector<int32_t> nonempty;  // indices into patches
    int32_t n_cells = 0, n_ifaces = 0, n_bfaces = 0;
    std::vector<double> V, C, Sf, Cf, magSf, w, delta, bSf, bCf, bmagSf, bw, bdelta;
    std::vector<int32_t> owner, neighbour, bcells, patch_offs;
};

extern "C" fvgb_status fvgb_polymesh_read(const char* dir, fvgb_polymesh** out, fvgb_mesh_desc* desc) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(dir && out && desc, "fvgb_polymesh_read: null argument");
    const std::string d = std::string(dir) + "/";
    auto pm = new fvgb_polymesh();
    auto fail = [&](fvgb_status st, const char* what) {
        delete pm;
        return fvgb_fail(st, what);
    };
    std::string text;
    bool binary = false;
    // points
    if (!read_text(d + "points", text)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: cannot read points");
    {
        Lexer lx{text};
        if (!skip_header(lx)) return fail(FVGB_ERR_UNSUPPORTED, "fvgb_polymesh_read: binary points");
        long n;
        if (!list_start(lx, n)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed points");
        pm->points.resize(3 * (size_t)n);
        std::string t;
        for (long k = 0; k < n; ++k) {
            if (!lx.expect("(")) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed point");
            for (int c = 0; c < 3; ++c)
                if (!lx.next(t) || !to_double(t, pm->points[3 * (size_t)k + c]))
                    return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed point");
            if (!lx.expect(")")) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed point");
        }
        if (!lx.expect(")")) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed points");
    }
    // faces
    std::vector<int32_t> foffs{0}, fpts;
    if (!read_text(d + "faces", text)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: cannot read faces");
    {
        Lexer lx{text};
        if (!skip_header(lx)) return fail(FVGB_ERR_UNSUPPORTED, "fvgb_polymesh_read: binary faces");
        long n;
        if (!list_start(lx, n)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed faces");
        std::string t;
        for (long k = 0; k < n; ++k) {
            long m;
            if (!list_start(lx, m) || m < 3) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed face");
            for (long q = 0; q < m; ++q) {
                long v;
                if (!lx.next(t) || !to_long(t, v) || v < 0 || 3 * (size_t)v >= pm->points.size())
                    return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: face point out of range");
                fpts.push_back((int32_t)v);
            }
            if (!lx.expect(")")) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed face");
            foffs.push_back((int32_t)fpts.size());
        }
    }
    const long n_faces = (long)foffs.size() - 1;
    std::vector<int32_t> owner_file, nei;
    if (!read_labels(d + "owner", owner_file, binary))
        return fail(binary ? FVGB_ERR_UNSUPPORTED : FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: owner");
    if (!read_labels(d + "neighbour", nei, binary))
        return fail(binary ? FVGB_ERR_UNSUPPORTED : FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: neighbour");
    if ((long)owner_file.size() != n_faces || (long)nei.size() > n_faces)
        return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: owner/neighbour sizes do not match faces");
    // boundary
    if (!read_text(d + "boundary", text)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: cannot read boundary");
    {
        Lexer lx{text};
        if (!skip_header(lx)) return fail(FVGB_ERR_UNSUPPORTED, "fvgb_polymesh_read: binary boundary");
        long n;
        if (!list_start(lx, n)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed boundary");
        std::string t;
        for (long k = 0; k < n; ++k) {
            Patch p;
            if (!lx.next(p.name) || !lx.expect("{")) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: patch");
            for (;;) {
                std::string key;
                if (!lx.next(key)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: patch");
                if (key == "}") break;
                std::string val, tok;
                int depth = 0;
                while (lx.next(tok) && !(tok == ";" && depth == 0)) {  // a value may be a list: 1(wall)
                    if (tok == "(") ++depth;
                    if (tok == ")") --depth;
                    if (val.empty()) val = tok;
                }
                if (key == "type") p.type = val;
                else if (key == "nFaces" && !to_long(val, p.n_faces)) return fail(FVGB_ERR_INVALID_ARG, "nFaces");
                else if (key == "startFace" && !to_long(val, p.start)) return fail(FVGB_ERR_INVALID_ARG, "startFace");
            }
            if (p.start < 0 || p.n_faces < 0 || p.start + p.n_faces > n_faces)
                return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: patch faces out of range");
            pm->patches.push_back(p);
        }
    }
    // internal faces first, then the non-empty patches in order; empty patches last (skipped)
    const int32_t nif = (int32_t)nei.size();
    std::vector<int32_t> order(nif), empties;
    for (int32_t f = 0; f < nif; ++f) order[f] = f;
    pm->patch_offs.push_back(0);
    for (size_t k = 0; k < pm->patches.size(); ++k) {
        const Patch& p = pm->patches[k];
        for (long f = p.start; f < p.start + p.n_faces; ++f) (p.type == "empty" ? empties : order).push_back((int32_t)f);
        if (p.type != "empty") {
            pm->nonempty.push_back((int32_t)k);
            pm->patch_offs.push_back((int32_t)(order.size() - nif));
        }
    }
    const int32_t nbf = (int32_t)order.size() - nif;
    std::vector<int32_t> perm = order;
    perm.insert(perm.end(), empties.begin(), empties.end());
    std::vector<int32_t> po{0}, pp, own;
    int32_t ncells = 0;
    for (int32_t f : perm) {
        for (int32_t q = foffs[f]; q < foffs[f + 1]; ++q) pp.push_back(fpts[q]);
        po.push_back((int32_t)pp.size());
        own.push_back(owner_file[f]);
        ncells = std::max(ncells, owner_file[f] + 1);
    }
    for (int32_t v : nei) ncells = std::max(ncells, v + 1);
    pm->n_cells = ncells;
    pm->n_ifaces = nif;
    pm->n_bfaces = nbf;
    auto sz = [](std::vector<double>& v, size_t n) { v.assign(n ? n : 1, 0.0); };
    sz(pm->V, ncells);
    sz(pm->C, 3 * (size_t)ncells);
    sz(pm->Sf, 3 * (size_t)nif);
    sz(pm->Cf, 3 * (size_t)nif);
    sz(pm->magSf, nif);
    sz(pm->w, nif);
    sz(pm->delta, nif);
    sz(pm->bSf, 3 * (size_t)nbf);
    sz(pm->bCf, 3 * (size_t)nbf);
    sz(pm->bmagSf, nbf);
    sz(pm->bw, nbf);
    sz(pm->bdelta, nbf);
    pm->owner.assign(own.begin(), own.begin() + nif);
    pm->neighbour = nei;
    pm->bcells.assign(nbf ? nbf : 1, 0);
    fvgb_mesh_arrays a{};
    a.cell_volumes = pm->V.data();
    a.cell_centres = pm->C.data();
    a.owner = nullptr;
    a.neighbour = nullptr;
    a.face_areas = pm->Sf.data();
    a.face_centres = pm->Cf.data();
    a.mag_face_areas = pm->magSf.data();
    a.weights = pm->w.data();
    a.delta_coeffs = pm->delta.data();
    a.bface_cells = pm->bcells.data();
    a.bface_areas = pm->bSf.data();
    a.bface_centres = pm->bCf.data();
    a.bmag_face_areas = pm->bmagSf.data();
    a.bweights = pm->bw.data();
    a.bdelta_coeffs = pm->bdelta.data();
    a.patch_offsets = nullptr;
    const int32_t npts = (int32_t)(pm->points.size() / 3);
    fvgb_status st = fvgb_geometry_compute(npts, pm->points.data(), ncells, (int32_t)perm.size(), po.data(),
                                           pp.data(), own.data(), nif, nei.data(), nbf, &a);
    if (st != FVGB_OK) {
        delete pm;
        return st;
    }
    fvgb_mesh_desc& m = *desc;
    m.n_cells = ncells;
    m.n_ifaces = nif;
    m.n_bfaces = nbf;
    m.n_patches = (int32_t)pm->nonempty.size();
    m.cell_volumes = pm->V.data();
    m.cell_centres = pm->C.data();
    m.owner = pm->owner.data();
    m.neighbour = pm->neighbour.data();
    m.face_areas = pm->Sf.data();
    m.mag_face_areas = pm->magSf.data();
    m.weights = pm->w.data();
    m.delta_coeffs = pm->delta.data();
    m.bface_cells = pm->bcells.data();
    m.bface_areas = pm->bSf.data();
    m.bmag_face_areas = pm->bmagSf.data();
    m.bweights = pm->bw.data();
    m.bdelta_coeffs = pm->bdelta.data();
    m.patch_offsets = pm->patch_offs.data();
    *out = pm;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_polymesh_patch(const fvgb_polymesh* pm, int32_t p, const char** name, const char** type) {
    FVGB_CHECK_ARG(pm && name && type, "fvgb_polymesh_patch: null argument");
    FVGB_CHECK_ARG(p >= 0 && p < (int32_t)pm->nonempty.size(), "fvgb_polymesh_patch: no such non-empty patch");
    const Patch& q = pm->patches[(size_t)pm->nonempty[(size_t)p]];
    *name = q.name.c_str();
    *type = q.type.c_str();
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_polymesh_free(fvgb_polymesh* pm) {
    delete pm;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_field_read(const char* path, int32_t n, double* values) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(path && values && n >= 0, "fvgb_field_read: bad argument");
    std::string text;
    if (!read_text(path, text)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_read: cannot read the file");
    Lexer lx{text};
    if (!skip_header(lx)) return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_field_read: binary field");
    std::string t;
    while (lx.next(t) && t != "internalField") {
    }
    if (t != "internalField" || !lx.next(t)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_read: no internalField");
    if (t == "uniform") {
        double v;
        if (!lx.next(t) || !to_double(t, v)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_read: uniform value");
        for (int32_t i = 0; i < n; ++i) values[i] = v;
        return FVGB_OK;
    }
    if (t != "nonuniform" || !lx.next(t) || t != "List<scalar>")
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "fvgb_field_read: internalField is not a scalar list");
    long m;
    if (!list_start(lx, m) || m != n) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_read: list size is not n");
    for (int32_t i = 0; i < n; ++i)
        if (!lx.next(t) || !to_double(t, values[i])) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_read: value");
    return lx.expect(")") ? FVGB_OK : fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_read: unterminated list");
}

extern "C" fvgb_status fvgb_field_write(const char* path, const char* object, const fvgb_polymesh* pm,
                                        const double* internal, const double* boundary) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(path && object && pm && internal && (boundary || pm->n_bfaces == 0),
                   "fvgb_field_write: null argument");
    FILE* f = std::fopen(path, "w");
    if (!f) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_write: cannot open the file");
    std::fprintf(f,
                 "FoamFile\n{\n    version     2.0;\n    format      ascii;\n    class       volScalarField;\n"
                 "    object      %s;\n}\n\ndimensions      [0 0 0 0 0 0 0];\n\n",
                 object);
    auto list = [&](const double* v, long n) {
        std::fprintf(f, "nonuniform List<scalar>\n%ld\n(\n", n);
        for (long i = 0; i < n; ++i) std::fprintf(f, "%.17g\n", v[i]);  // round-trips every double
        std::fprintf(f, ")\n");
    };
    std::fprintf(f, "internalField   ");
    list(internal, pm->n_cells);
    std::fprintf(f, ";\n\nboundaryField\n{\n");
    int32_t q = 0;
    for (size_t k = 0; k < pm->patches.size(); ++k) {
        const Patch& p = pm->patches[k];
        std::fprintf(f, "    %s\n    {\n", p.name.c_str());
        if (p.type == "empty") {
            std::fprintf(f, "        type            empty;\n");
        } else {
            std::fprintf(f, "        type            calculated;\n        value           ");
            const int32_t b0 = pm->patch_offs[(size_t)q], b1 = pm->patch_offs[(size_t)q + 1];
            list(boundary + b0, b1 - b0);
            std::fprintf(f, "        ;\n");
            ++q;
        }
        std::fprintf(f, "    }\n");
    }
    std::fprintf(f, "}\n");
    const bool ok = std::fclose(f) == 0;
    return ok ? FVGB_OK : fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_write: write failed");
}
