// OpenFOAM files on the host: the polyMesh a case is read from, the field
// files its initial and boundary conditions come from, and the field files
// results are written to, in the ascii and the binary format.  In FoamAdapter
// these are the steps before and after the hot path: MeshAdapter builds the
// NeoN mesh from Foam::fvMesh (src/datastructures/meshAdapter.cpp:59-136),
// readVolBoundaryConditions maps the boundaryField entries to NeoN boundary
// conditions (include/FoamAdapter/auxiliary/readers.hpp:31-108) and
// writers.cpp:9-135 writes NeoN fields back as OpenFOAM fields.  Geometry is
// computed by fvgb_geometry_compute (meshgen.cpp), the same routine the box
// builder uses.
//
// Binary files follow OpenFOAM's layout: the FoamFile header and every
// keyword are text; a list is "N(" followed by N items of raw little-endian
// bytes and ")", with the label and scalar widths declared by the header's
// arch entry ("LSB;label=32;scalar=64"); a faces file is a faceCompactList
// (offsets [nFaces+1], then the concatenated point labels).
#include <algorithm>
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <regex>
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
// List<scalar>), quoted strings and the punctuation ( ) { } ; -- comments
// removed.  raw() takes the bytes of a binary list body.
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
        if (s[i] == '"') {
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
    bool raw(void* dst, size_t bytes) {
        if (i > s.size() || bytes > s.size() - i) return false;
        if (bytes) std::memcpy(dst, s.data() + i, bytes);
        i += bytes;
        return true;
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

struct Format {
    bool binary = false;
    int label_bytes = 4, scalar_bytes = 8;
    std::string cls;
};

bool host_little_endian() {
    const uint16_t one = 1;
    uint8_t b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

// The FoamFile header, if any: format, arch and class.  Returns
// FVGB_ERR_UNSUPPORTED for a big-endian arch or label/scalar widths other than
// 32/64 bits, FVGB_ERR_INVALID_ARG for an unterminated header.
fvgb_status read_header(Lexer& lx, Format& fmt) {
    const size_t save = lx.i;
    std::string t;
    if (!lx.next(t) || t != "FoamFile") {
        lx.i = save;
        return FVGB_OK;
    }
    if (!lx.expect("{")) return FVGB_ERR_INVALID_ARG;
    std::string key;
    for (;;) {
        if (!lx.next(key)) return FVGB_ERR_INVALID_ARG;
        if (key == "}") break;
        std::string val, tok;
        while (lx.next(tok) && tok != ";")
            if (val.empty()) val = tok;
        if (key == "format") {
            fmt.binary = val == "binary";
        } else if (key == "class") {
            fmt.cls = val;
        } else if (key == "arch") {
            if (val.find("MSB") != std::string::npos) return FVGB_ERR_UNSUPPORTED;
            const size_t l = val.find("label="), s = val.find("scalar=");
            if (l != std::string::npos) fmt.label_bytes = std::atoi(val.c_str() + l + 6) / 8;
            if (s != std::string::npos) fmt.scalar_bytes = std::atoi(val.c_str() + s + 7) / 8;
        }
    }
    if (fmt.label_bytes != 4 && fmt.label_bytes != 8) return FVGB_ERR_UNSUPPORTED;
    if (fmt.scalar_bytes != 4 && fmt.scalar_bytes != 8) return FVGB_ERR_UNSUPPORTED;
    if (fmt.binary && !host_little_endian()) return FVGB_ERR_UNSUPPORTED;
    return FVGB_OK;
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

bool read_count(Lexer& lx, long& n) {
    std::string t;
    return lx.next(t) && to_long(t, n) && n >= 0;
}

// One item of ncomp numbers in text: "v" or "(x y z)".
bool read_item_text(Lexer& lx, int ncomp, double* v) {
    std::string t;
    if (ncomp == 1) return lx.next(t) && to_double(t, v[0]);
    if (!lx.expect("(")) return false;
    for (int c = 0; c < ncomp; ++c)
        if (!lx.next(t) || !to_double(t, v[c])) return false;
    return lx.expect(")");
}

bool read_scalar_raw(Lexer& lx, const Format& fmt, size_t m, double* out) {
    if (fmt.scalar_bytes == 8) return lx.raw(out, m * 8);
    std::vector<float> f(m);
    if (!lx.raw(f.data(), m * 4)) return false;
    for (size_t k = 0; k < m; ++k) out[k] = f[k];
    return true;
}

// The body of a list of n items of ncomp scalars, its count already read:
// "( ... )" in text or raw bytes, or the uniform form "{ item }".
bool read_scalar_body(Lexer& lx, const Format& fmt, int ncomp, long n, std::vector<double>& out) {
    out.assign((size_t)n * ncomp, 0.0);
    std::string t;
    if (!lx.next(t)) return false;
    if (t == "{") {
        double v[3] = {0, 0, 0};  // the uniform form is text in both formats
        if (!read_item_text(lx, ncomp, v)) return false;
        for (long k = 0; k < n; ++k)
            for (int c = 0; c < ncomp; ++c) out[(size_t)k * ncomp + c] = v[c];
        return lx.expect("}");
    }
    if (t != "(") return false;
    if (fmt.binary) {
        if (!read_scalar_raw(lx, fmt, out.size(), out.data())) return false;
    } else {
        for (long k = 0; k < n; ++k)
            if (!read_item_text(lx, ncomp, out.data() + (size_t)k * ncomp)) return false;
    }
    return lx.expect(")");
}

bool label_ok(long long v) { return v >= -1 && v <= 0x7fffffffLL; }

// The body of a list of n labels (count already read); 64-bit labels must fit int32.
bool read_label_body(Lexer& lx, const Format& fmt, long n, std::vector<int32_t>& out) {
    out.assign((size_t)n, 0);
    std::string t;
    if (!lx.next(t)) return false;
    auto raw_one = [&](long long& v) {
        if (fmt.label_bytes == 4) {
            int32_t x;
            if (!lx.raw(&x, 4)) return false;
            v = x;
        } else {
            int64_t x;
            if (!lx.raw(&x, 8)) return false;
            v = x;
        }
        return label_ok(v);
    };
    auto text_one = [&](long long& v) {
        long x;
        if (!lx.next(t) || !to_long(t, x)) return false;
        v = x;
        return label_ok(v);
    };
    if (t == "{") {
        long long v;  // the uniform form is text in both formats
        if (!text_one(v)) return false;
        std::fill(out.begin(), out.end(), (int32_t)v);
        return lx.expect("}");
    }
    if (t != "(") return false;
    for (long k = 0; k < n; ++k) {
        long long v;
        if (!(fmt.binary ? raw_one(v) : text_one(v))) return false;
        out[(size_t)k] = (int32_t)v;
    }
    return lx.expect(")");
}

// A file holding one top-level list after its header.
fvgb_status open_list(const std::string& path, std::string& text, Lexer& lx, Format& fmt, long& n) {
    if (!read_text(path, text)) return FVGB_ERR_INVALID_ARG;
    lx = Lexer{text};
    const fvgb_status st = read_header(lx, fmt);
    if (st != FVGB_OK) return st;
    return read_count(lx, n) ? FVGB_OK : FVGB_ERR_INVALID_ARG;
}

// Tokens of an entry's value up to its ';' (nested ( ) and { } kept whole);
// a value that is a sub-dictionary ends with its closing brace.
bool entry_tokens(Lexer& lx, std::vector<std::string>& toks) {
    toks.clear();
    int depth = 0;
    std::string t;
    while (lx.next(t)) {
        if (t == ";" && depth == 0) return true;
        if (t == "(" || t == "{") ++depth;
        if (t == ")" || t == "}") --depth;
        toks.push_back(t);
        if (depth == 0 && t == "}" && toks.front() == "{") return true;
    }
    return false;
}

struct Patch {
    std::string name, type;
    std::vector<std::string> groups;
    long n_faces = 0, start = 0;
};

// A field value entry: "uniform item", "nonuniform List<T> N(...)" (text or
// binary), or something else (kept as words).
struct Value {
    enum Kind { NONE, UNIFORM, NONUNIFORM, OTHER } kind = NONE;
    std::vector<double> data;  // UNIFORM: ncomp numbers; NONUNIFORM: n*ncomp
    std::vector<std::string> words;
};

fvgb_status read_value(Lexer& lx, const Format& fmt, int ncomp, Value& v, const Value* internal) {
    std::string t;
    const size_t save = lx.i;
    if (!lx.next(t)) return FVGB_ERR_INVALID_ARG;
    if (t == "uniform") {
        v.kind = Value::UNIFORM;
        v.data.assign((size_t)ncomp, 0.0);
        if (!read_item_text(lx, ncomp, v.data.data())) return FVGB_ERR_INVALID_ARG;
        return lx.expect(";") ? FVGB_OK : FVGB_ERR_INVALID_ARG;
    }
    if (t == "nonuniform") {
        if (!lx.next(t)) return FVGB_ERR_INVALID_ARG;
        const char* want = ncomp == 1 ? "List<scalar>" : "List<vector>";
        if (t != want) return FVGB_ERR_UNSUPPORTED;
        long n;
        if (!read_count(lx, n) || !read_scalar_body(lx, fmt, ncomp, n, v.data)) return FVGB_ERR_INVALID_ARG;
        v.kind = Value::NONUNIFORM;
        return lx.expect(";") ? FVGB_OK : FVGB_ERR_INVALID_ARG;
    }
    if (t == "$internalField" && internal && internal->kind == Value::UNIFORM) {
        v = *internal;
        return lx.expect(";") ? FVGB_OK : FVGB_ERR_INVALID_ARG;
    }
    lx.i = save;
    v.kind = Value::OTHER;
    return entry_tokens(lx, v.words) ? FVGB_OK : FVGB_ERR_INVALID_ARG;
}

// A volume/surface field file: internalField and each boundaryField entry.
struct FieldFile {
    Format fmt;
    Value internal;
    struct Entry {
        std::string key;  // patch name, group name or quoted regular expression
        std::string type;
        Value value;
    };
    std::vector<Entry> patches;
};

fvgb_status parse_field(const char* path, int ncomp, FieldFile& ff) {
    std::string text;
    if (!read_text(path, text)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "field file: cannot read the file");
    Lexer lx{text};
    fvgb_status st = read_header(lx, ff.fmt);
    if (st != FVGB_OK) return fvgb_fail(st, "field file: header");
    std::string key;
    while (lx.next(key)) {
        if (key == "internalField") {
            st = read_value(lx, ff.fmt, ncomp, ff.internal, nullptr);
            if (st != FVGB_OK) return fvgb_fail(st, "field file: internalField");
        } else if (key == "boundaryField") {
            if (!lx.expect("{")) return fvgb_fail(FVGB_ERR_INVALID_ARG, "field file: boundaryField");
            for (;;) {
                std::string name;
                if (!lx.next(name)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "field file: unterminated boundaryField");
                if (name == "}") break;
                if (name[0] == '#') {  // #includeEtc "..." and the like: ignored
                    std::string arg;
                    lx.next(arg);
                    continue;
                }
                if (!lx.expect("{")) return fvgb_fail(FVGB_ERR_INVALID_ARG, "field file: patch entry");
                FieldFile::Entry e;
                e.key = name;
                for (;;) {
                    std::string k;
                    if (!lx.next(k)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "field file: unterminated patch entry");
                    if (k == "}") break;
                    Value v;
                    st = read_value(lx, ff.fmt, ncomp, v, &ff.internal);
                    if (st != FVGB_OK) return fvgb_fail(st, "field file: patch value");
                    if (k == "type" && v.kind == Value::OTHER && !v.words.empty()) e.type = v.words[0];
                    else if (k == "value") e.value = v;
                }
                ff.patches.push_back(e);
            }
        } else if (key == ";") {
        } else if (key[0] == '#') {  // #include "file" and the like: ignored
            std::string arg;
            lx.next(arg);
        } else {
            std::vector<std::string> toks;  // dimensions [...] and other top-level entries
            if (!entry_tokens(lx, toks)) break;
        }
    }
    if (ff.internal.kind != Value::UNIFORM && ff.internal.kind != Value::NONUNIFORM)
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "field file: no internalField");
    return FVGB_OK;
}

}  // namespace

struct fvgb_polymesh {
    std::vector<double> points;
    std::vector<Patch> patches;     // every patch, in file order
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
    Lexer lx;
    fvgb_status st;
    long n;
    // points: vectorField
    {
        Format fmt;
        if ((st = open_list(d + "points", text, lx, fmt, n)) != FVGB_OK) return fail(st, "fvgb_polymesh_read: points");
        if (!read_scalar_body(lx, fmt, 3, n, pm->points)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: points");
    }
    const long npts = (long)pm->points.size() / 3;
    // faces: faceList (text) or faceCompactList (text or binary)
    std::vector<int32_t> foffs, fpts;
    {
        Format fmt;
        if ((st = open_list(d + "faces", text, lx, fmt, n)) != FVGB_OK) return fail(st, "fvgb_polymesh_read: faces");
        if (fmt.cls == "faceCompactList") {
            long m;
            if (n < 1 || !read_label_body(lx, fmt, n, foffs) || !read_count(lx, m) || !read_label_body(lx, fmt, m, fpts))
                return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: faces");
            if (foffs[0] != 0 || foffs.back() != (int32_t)m)
                return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: face offsets");
            for (size_t k = 0; k + 1 < foffs.size(); ++k)
                if (foffs[k + 1] - foffs[k] < 3) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: face offsets");
        } else {
            if (fmt.binary) return fail(FVGB_ERR_UNSUPPORTED, "fvgb_polymesh_read: binary faces must be a faceCompactList");
            if (!lx.expect("(")) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: faces");
            foffs.push_back(0);
            std::vector<int32_t> one;
            for (long k = 0; k < n; ++k) {
                long m;
                if (!read_count(lx, m) || m < 3 || !read_label_body(lx, fmt, m, one))
                    return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: malformed face");
                fpts.insert(fpts.end(), one.begin(), one.end());
                foffs.push_back((int32_t)fpts.size());
            }
            if (!lx.expect(")")) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: faces");
        }
        for (int32_t v : fpts)
            if (v < 0 || v >= npts) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: face point out of range");
    }
    const long n_faces = (long)foffs.size() - 1;
    std::vector<int32_t> owner_file, nei;
    {
        Format fmt;
        if ((st = open_list(d + "owner", text, lx, fmt, n)) != FVGB_OK || !read_label_body(lx, fmt, n, owner_file))
            return fail(st != FVGB_OK ? st : FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: owner");
    }
    {
        Format fmt;
        if ((st = open_list(d + "neighbour", text, lx, fmt, n)) != FVGB_OK || !read_label_body(lx, fmt, n, nei))
            return fail(st != FVGB_OK ? st : FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: neighbour");
        while (!nei.empty() && nei.back() < 0) nei.pop_back();  // a neighbour list padded to nFaces
    }
    if ((long)owner_file.size() != n_faces || (long)nei.size() > n_faces)
        return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: owner/neighbour sizes do not match faces");
    for (int32_t v : owner_file)
        if (v < 0) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: negative owner");
    for (int32_t v : nei)
        if (v < 0) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: negative neighbour");
    // boundary: a dictionary list, text in either format
    {
        Format fmt;
        if ((st = open_list(d + "boundary", text, lx, fmt, n)) != FVGB_OK || !lx.expect("("))
            return fail(st != FVGB_OK ? st : FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: boundary");
        for (long k = 0; k < n; ++k) {
            Patch p;
            if (!lx.next(p.name) || !lx.expect("{")) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: patch");
            for (;;) {
                std::string key;
                std::vector<std::string> toks;
                if (!lx.next(key)) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: patch");
                if (key == "}") break;
                if (!entry_tokens(lx, toks) || toks.empty()) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: patch");
                if (key == "type") {
                    p.type = toks[0];
                } else if (key == "nFaces" && !to_long(toks[0], p.n_faces)) {
                    return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: nFaces");
                } else if (key == "startFace" && !to_long(toks[0], p.start)) {
                    return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: startFace");
                } else if (key == "inGroups") {  // N(a b ...)
                    for (size_t q = 1; q < toks.size(); ++q)
                        if (toks[q] != "(" && toks[q] != ")") p.groups.push_back(toks[q]);
                }
            }
            if (p.start < 0 || p.n_faces < 0 || p.start + p.n_faces > n_faces)
                return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: patch faces out of range");
            pm->patches.push_back(p);
        }
    }
    // internal faces first, then the non-empty patches in order; empty patches
    // (fvPatch size 0) last and left out of the flat boundary
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
    if ((long)perm.size() != n_faces) return fail(FVGB_ERR_INVALID_ARG, "fvgb_polymesh_read: patches do not cover the boundary faces");
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
    auto sz = [](std::vector<double>& v, size_t k) { v.assign(k ? k : 1, 0.0); };
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
    st = fvgb_geometry_compute((int32_t)npts, pm->points.data(), ncells, (int32_t)perm.size(), po.data(), pp.data(),
                               own.data(), nif, nei.data(), nbf, &a);
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
    fvgb_clear_error();
    FVGB_CHECK_ARG(pm && name && type, "fvgb_polymesh_patch: null argument");
    FVGB_CHECK_ARG(p >= 0 && p < (int32_t)pm->nonempty.size(), "fvgb_polymesh_patch: no such non-empty patch");
    const Patch& q = pm->patches[(size_t)pm->nonempty[(size_t)p]];
    *name = q.name.c_str();
    *type = q.type.c_str();
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_polymesh_geometry(const fvgb_polymesh* pm, int32_t* n_points, const double** points,
                                              const double** face_centres, const double** bface_centres) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(pm && n_points && points && face_centres && bface_centres, "fvgb_polymesh_geometry: null argument");
    *n_points = (int32_t)(pm->points.size() / 3);
    *points = pm->points.data();
    *face_centres = pm->Cf.data();
    *bface_centres = pm->bCf.data();
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_polymesh_free(fvgb_polymesh* pm) {
    delete pm;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_field_read(const char* path, int32_t n, int32_t ncomp, double* values) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(path && (values || n == 0) && n >= 0, "fvgb_field_read: bad argument");
    FVGB_CHECK_ARG(ncomp == 1 || ncomp == 3, "fvgb_field_read: ncomp must be 1 or 3");
    FieldFile ff;
    const fvgb_status st = parse_field(path, ncomp, ff);
    if (st != FVGB_OK) return st;
    const Value& v = ff.internal;
    if (v.kind == Value::UNIFORM) {
        for (int32_t i = 0; i < n; ++i)
            for (int c = 0; c < ncomp; ++c) values[(size_t)i * ncomp + c] = v.data[(size_t)c];
        return FVGB_OK;
    }
    if (v.data.size() != (size_t)n * ncomp) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_read: list size is not n");
    std::copy(v.data.begin(), v.data.end(), values);
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_field_read_bc(const char* path, const fvgb_polymesh* pm, int32_t ncomp,
                                          int32_t* patch_type, double* ref, double* boundary) {
    fvgb_clear_error();
    FVGB_CHECK_ARG(path && pm && patch_type && (ref || pm->n_bfaces == 0), "fvgb_field_read_bc: null argument");
    FVGB_CHECK_ARG(ncomp == 1 || ncomp == 3, "fvgb_field_read_bc: ncomp must be 1 or 3");
    FieldFile ff;
    fvgb_status st = parse_field(path, ncomp, ff);
    if (st != FVGB_OK) return st;
    // entry of a patch: its own name, then a group it is in, then a quoted
    // regular expression matching its name (the order OpenFOAM resolves them)
    auto find = [&](const Patch& p) -> const FieldFile::Entry* {
        for (const auto& e : ff.patches)
            if (e.key == p.name) return &e;
        for (const auto& e : ff.patches)
            if (std::find(p.groups.begin(), p.groups.end(), e.key) != p.groups.end()) return &e;
        for (const auto& e : ff.patches) {
            if (e.key.size() < 2 || e.key.front() != '"') continue;
            try {
                if (std::regex_match(p.name, std::regex(e.key.substr(1, e.key.size() - 2), std::regex::extended)))
                    return &e;
            } catch (const std::regex_error&) {
            }
        }
        return nullptr;
    };
    const size_t nb = (size_t)pm->n_bfaces * ncomp;
    std::fill(ref, ref + nb, 0.0);
    if (boundary) std::fill(boundary, boundary + nb, 0.0);
    for (size_t q = 0; q < pm->nonempty.size(); ++q) {
        const Patch& p = pm->patches[(size_t)pm->nonempty[q]];
        const FieldFile::Entry* e = find(p);
        if (!e) return fvgb_fail(FVGB_ERR_INVALID_ARG, ("fvgb_field_read_bc: no entry for patch " + p.name).c_str());
        const size_t b0 = (size_t)pm->patch_offs[q] * ncomp, b1 = (size_t)pm->patch_offs[q + 1] * ncomp;
        // the patch's `value` entry, per face
        auto fill = [&](const Value& v, double* dst) -> bool {
            if (v.kind == Value::UNIFORM) {
                for (size_t k = b0; k < b1; ++k) dst[k] = v.data[(k - b0) % ncomp];
                return true;
            }
            if (v.kind == Value::NONUNIFORM && v.data.size() == b1 - b0) {
                std::copy(v.data.begin(), v.data.end(), dst + b0);
                return true;
            }
            return false;
        };
        if (boundary) fill(e->value, boundary);
        // the mapping of readVolBoundaryConditions (readers.hpp:43-95)
        if (e->type == "fixedValue") {
            patch_type[q] = FVGB_BC_FIXED_VALUE;
            if (!fill(e->value, ref))
                return fvgb_fail(FVGB_ERR_INVALID_ARG, ("fvgb_field_read_bc: fixedValue without value: " + p.name).c_str());
        } else if (e->type == "fixedGradient") {
            // the reference takes the gradient from the patch's `value` entry (readers.hpp:45-50)
            patch_type[q] = FVGB_BC_FIXED_GRADIENT;
            if (!fill(e->value, ref))
                return fvgb_fail(FVGB_ERR_INVALID_ARG, ("fvgb_field_read_bc: fixedGradient without value: " + p.name).c_str());
        } else if (e->type == "zeroGradient") {
            patch_type[q] = FVGB_BC_FIXED_GRADIENT;
        } else if (e->type == "noSlip") {
            patch_type[q] = FVGB_BC_FIXED_VALUE;
        } else if (e->type == "calculated" || e->type == "extrapolatedCalculated") {
            patch_type[q] = FVGB_BC_CALCULATED;
        } else {
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, ("fvgb_field_read_bc: boundary condition " + e->type).c_str());
        }
    }
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_field_write(const char* path, const char* object, const fvgb_polymesh* pm, int32_t ncomp,
                                        const double* internal, const double* boundary, int32_t flags) {
    fvgb_clear_error();
    const bool surface = (flags & FVGB_IO_SURFACE) != 0, binary = (flags & FVGB_IO_BINARY) != 0;
    const int32_t n_int = surface ? pm->n_ifaces : pm->n_cells;
    FVGB_CHECK_ARG(path && object && pm && (internal || n_int == 0) && (boundary || pm->n_bfaces == 0),
                   "fvgb_field_write: null argument");
    FVGB_CHECK_ARG(ncomp == 1 || ncomp == 3, "fvgb_field_write: ncomp must be 1 or 3");
    FVGB_CHECK_ARG(!binary || host_little_endian(), "fvgb_field_write: binary output needs a little-endian host");
    FILE* f = std::fopen(path, "wb");
    if (!f) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_write: cannot open the file");
    const char* kind = ncomp == 1 ? "Scalar" : "Vector";
    std::fprintf(f,
                 "FoamFile\n{\n    version     2.0;\n    format      %s;\n    arch        \"LSB;label=32;scalar=64\";\n"
                 "    class       %s%sField;\n    object      %s;\n}\n\ndimensions      [0 0 0 0 0 0 0];\n\n",
                 binary ? "binary" : "ascii", surface ? "surface" : "vol", kind, object);
    auto list = [&](const double* v, long n) {
        std::fprintf(f, "nonuniform List<%s> %ld\n(", ncomp == 1 ? "scalar" : "vector", n);
        if (binary) {
            std::fwrite(v, sizeof(double), (size_t)n * ncomp, f);
        } else {
            std::fprintf(f, "\n");
            for (long i = 0; i < n; ++i) {  // %.17g round-trips every double
                if (ncomp == 1) std::fprintf(f, "%.17g\n", v[i]);
                else std::fprintf(f, "(%.17g %.17g %.17g)\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
            }
        }
        std::fprintf(f, ")\n");
    };
    std::fprintf(f, "internalField   ");
    list(internal, n_int);
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
            list(boundary + (size_t)b0 * ncomp, b1 - b0);
            std::fprintf(f, "        ;\n");
            ++q;
        }
        std::fprintf(f, "    }\n");
    }
    std::fprintf(f, "}\n");
    const bool ok = !std::ferror(f);
    return std::fclose(f) == 0 && ok ? FVGB_OK : fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_field_write: write failed");
}
