// OpenFOAM dictionaries on the host: system/fvSolution, system/fvSchemes and
// the like, read into a tree of entries, and the mapping FoamAdapter applies
// to an OpenFOAM solver entry before it hands it to NeoN/Ginkgo.
//
// In FoamAdapter, OpenFOAM parses the files (Foam::dictionary) and
// FoamAdapter::convert turns each entry into a NeoN::Dictionary value
// (src/auxiliary/foamDictionary.cpp:12-91, src/auxiliary/convert.cpp:17-45);
// mapFvSolution rewrites a solver entry into Ginkgo terms
// (src/compatibility/fvSolution.cpp:19-159).  Without OpenFOAM, this file
// parses the dictionary syntax itself and keeps each primitive entry as its
// token list; the typed views of the reference (label, scalar, vector, word,
// token list) are taken on the token lists by the host mirrors.
//
// Syntax: keyword value; entries, keyword { ... } sub-dictionaries, lists
// "( ... )" inside values, // and /* */ comments, quoted strings, words with
// balanced parentheses (div(phi,T) is one word), #include "file" (relative to
// the including file; also #includeIfPresent, #sinclude), #inputMode and
// #remove, $name in a value (the tokens of the entry name, looked up in the
// enclosing dictionaries from the innermost outwards) and $name; as an entry
// (the entries of the sub-dictionary name merged in).  A quoted keyword is a
// regular expression; a lookup tries the plain keywords first, then the
// patterns from the last one defined.  A repeated keyword merges
// sub-dictionaries and replaces primitive entries (OpenFOAM's default
// inputMode merge).  The FoamFile header is dropped, as OpenFOAM does.
// Directives that run code (#calc, #codeStream, #eval, #includeFunc,
// #includeEtc) return FVGB_ERR_UNSUPPORTED.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <regex>
#include <sstream>
#include <string>
#include <vector>

#include "fvgb.h"
#include "fvgb_host_common.h"
#include "json_min.h"

namespace {

struct Tok {
    int32_t kind = FVGB_TOK_WORD;
    std::string text;
    int64_t label = 0;
    double scalar = 0.0;
};

}  // namespace

struct fvgb_dict {
    struct Entry {
        std::string key;
        bool pattern = false;
        std::unique_ptr<fvgb_dict> sub;
        std::vector<Tok> toks;
    };
    std::vector<Entry> entries;
    fvgb_dict* parent = nullptr;
    bool top = false;
};

namespace {

// ---------------------------------------------------------------- entries
bool regex_full_match(const std::string& pattern, const std::string& key) {
    try {
        return std::regex_match(key, std::regex(pattern));
    } catch (const std::regex_error&) {
        return false;
    }
}

// Index of the entry a lookup of `key` finds: a plain keyword equal to it,
// else the last-defined pattern that matches it; -1 if none.
int find_entry(const fvgb_dict* d, const std::string& key) {
    for (size_t i = 0; i < d->entries.size(); ++i)
        if (!d->entries[i].pattern && d->entries[i].key == key) return (int)i;
    for (size_t k = d->entries.size(); k-- > 0;)
        if (d->entries[k].pattern && regex_full_match(d->entries[k].key, key)) return (int)k;
    return -1;
}

// Index of the entry stored under exactly this keyword (plain or pattern).
int find_exact(const fvgb_dict* d, const std::string& key, bool pattern) {
    for (size_t i = 0; i < d->entries.size(); ++i)
        if (d->entries[i].pattern == pattern && d->entries[i].key == key) return (int)i;
    return -1;
}

std::unique_ptr<fvgb_dict> deep_copy(const fvgb_dict* src, fvgb_dict* parent) {
    auto d = std::make_unique<fvgb_dict>();
    d->parent = parent;
    for (const auto& e : src->entries) {
        fvgb_dict::Entry c;
        c.key = e.key;
        c.pattern = e.pattern;
        c.toks = e.toks;
        if (e.sub) c.sub = deep_copy(e.sub.get(), d.get());
        d->entries.push_back(std::move(c));
    }
    return d;
}

void merge_into(fvgb_dict* dst, const fvgb_dict* src);

// Set dst[key] to a copy of a primitive entry (replacing) or merge a
// sub-dictionary into an existing one.
void put_entry(fvgb_dict* dst, const fvgb_dict::Entry& e) {
    const int at = find_exact(dst, e.key, e.pattern);
    if (e.sub) {
        if (at >= 0 && dst->entries[at].sub) {
            merge_into(dst->entries[at].sub.get(), e.sub.get());
            return;
        }
        fvgb_dict::Entry c;
        c.key = e.key;
        c.pattern = e.pattern;
        c.sub = deep_copy(e.sub.get(), dst);
        if (at >= 0) dst->entries[at] = std::move(c);
        else dst->entries.push_back(std::move(c));
        return;
    }
    fvgb_dict::Entry c;
    c.key = e.key;
    c.pattern = e.pattern;
    c.toks = e.toks;
    if (at >= 0) dst->entries[at] = std::move(c);
    else dst->entries.push_back(std::move(c));
}

void merge_into(fvgb_dict* dst, const fvgb_dict* src) {
    for (const auto& e : src->entries) put_entry(dst, e);
}

// $name: the entry a lookup finds in d or, failing that, in the dictionaries
// enclosing it, innermost first.
const fvgb_dict::Entry* find_scoped(const fvgb_dict* d, const std::string& name) {
    for (const fvgb_dict* s = d; s; s = s->parent) {
        const int i = find_entry(s, name);
        if (i >= 0) return &s->entries[i];
    }
    return nullptr;
}

// ---------------------------------------------------------------- tokens
Tok classify(const std::string& w) {
    Tok t;
    t.text = w;
    t.kind = FVGB_TOK_WORD;
    if (w.empty()) return t;
    const char* s = w.c_str();
    char* end = nullptr;
    size_t k = (s[0] == '+' || s[0] == '-') ? 1 : 0;
    bool digits = k < w.size();
    for (size_t j = k; j < w.size(); ++j)
        if (!std::isdigit((unsigned char)w[j])) digits = false;
    if (digits) {
        errno = 0;
        const long long v = std::strtoll(s, &end, 10);
        if (errno == 0 && end && *end == '\0') {
            t.kind = FVGB_TOK_LABEL;
            t.label = (int64_t)v;
            t.scalar = (double)v;
            return t;
        }
    }
    if (std::isdigit((unsigned char)s[k]) || (s[k] == '.' && k + 1 < w.size() && std::isdigit((unsigned char)s[k + 1]))) {
        errno = 0;
        const double v = std::strtod(s, &end);
        if (end && *end == '\0' && errno != ERANGE) {
            t.kind = FVGB_TOK_SCALAR;
            t.scalar = v;
        }
    }
    return t;
}

struct Lex {
    std::string s;
    size_t i = 0;
    static bool punct(char c) { return c == '{' || c == '}' || c == ';' || c == '(' || c == ')' || c == '[' || c == ']'; }
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
    // kind: 0 end, 1 punctuation, 2 word, 3 quoted string (text without quotes)
    int next(std::string& t) {
        skip();
        if (i >= s.size()) return 0;
        const char c = s[i];
        if (c == '"') {
            std::string out;
            ++i;
            while (i < s.size() && s[i] != '"') {
                if (s[i] == '\\' && i + 1 < s.size()) ++i;
                out.push_back(s[i++]);
            }
            if (i >= s.size()) return -1;  // unterminated string
            ++i;
            t = out;
            return 3;
        }
        if (punct(c)) {
            t.assign(1, c);
            ++i;
            return 1;
        }
        // a word; parentheses inside it are kept while they balance
        const size_t b = i;
        int depth = 0;
        while (i < s.size()) {
            const char d = s[i];
            if (std::isspace((unsigned char)d)) break;
            if (d == '(') {
                ++depth;
            } else if (d == ')') {
                if (depth == 0) break;
                --depth;
            } else if (d == '{' || d == '}' || d == ';' || d == '[' || d == ']') {
                break;
            } else if (d == '"' && depth == 0) {
                break;
            }
            ++i;
        }
        t = s.substr(b, i - b);
        return 2;
    }
    size_t save() const { return i; }
    void restore(size_t p) { i = p; }
};

bool read_file(const std::string& path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

std::string dir_of(const std::string& path) {
    const size_t p = path.find_last_of('/');
    return p == std::string::npos ? std::string(".") : path.substr(0, p);
}

struct Parser {
    std::string err;
    int status = FVGB_OK;
    int depth_files = 0;

    bool fail(int st, const std::string& msg) {
        if (status == FVGB_OK) {
            status = st;
            err = msg;
        }
        return false;
    }

    // Tokens of a primitive entry up to its ';' (balanced parentheses), with
    // $name tokens replaced by the tokens of the entry they name.
    bool read_value(Lex& lx, fvgb_dict* d, std::vector<Tok>& out) {
        int depth = 0;
        std::string t;
        for (;;) {
            const int k = lx.next(t);
            if (k == 0) return fail(FVGB_ERR_INVALID_ARG, "dictionary: missing ';' at the end of input");
            if (k < 0) return fail(FVGB_ERR_INVALID_ARG, "dictionary: unterminated string");
            if (k == 1) {
                if (t == ";" && depth == 0) return true;
                if (t == "{" || t == "}") {
                    if (depth == 0) return fail(FVGB_ERR_INVALID_ARG, "dictionary: unexpected '" + t + "' in a value");
                }
                if (t == "(" || t == "[") ++depth;
                if (t == ")" || t == "]") {
                    if (depth == 0) return fail(FVGB_ERR_INVALID_ARG, "dictionary: unbalanced ')' in a value");
                    --depth;
                }
                Tok p;
                p.kind = FVGB_TOK_PUNCT;
                p.text = t;
                out.push_back(p);
                continue;
            }
            if (k == 3) {
                Tok q;
                q.kind = FVGB_TOK_STRING;
                q.text = t;
                out.push_back(q);
                continue;
            }
            if (t.size() > 1 && t[0] == '$') {
                const std::string name = t.substr(1);
                const fvgb_dict::Entry* e = find_scoped(d, name);
                if (!e) return fail(FVGB_ERR_INVALID_ARG, "dictionary: undefined variable $" + name);
                if (e->sub) return fail(FVGB_ERR_UNSUPPORTED, "dictionary: $" + name + " names a sub-dictionary inside a value");
                out.insert(out.end(), e->toks.begin(), e->toks.end());
                continue;
            }
            out.push_back(classify(t));
        }
    }

    bool include(const std::string& path, fvgb_dict* d, bool optional) {
        std::string text;
        if (!read_file(path, text)) {
            if (optional) return true;
            return fail(FVGB_ERR_INVALID_ARG, "dictionary: cannot read included file " + path);
        }
        if (++depth_files > 32) return fail(FVGB_ERR_INVALID_ARG, "dictionary: #include nested too deeply");
        Lex lx;
        lx.s = std::move(text);
        const bool ok = body(lx, d, dir_of(path), false);
        --depth_files;
        return ok;
    }

    // Entries up to the closing '}' (closed) or the end of the input.
    bool body(Lex& lx, fvgb_dict* d, const std::string& dir, bool closed) {
        std::string t;
        for (;;) {
            const int k = lx.next(t);
            if (k < 0) return fail(FVGB_ERR_INVALID_ARG, "dictionary: unterminated string");
            if (k == 0) {
                if (closed) return fail(FVGB_ERR_INVALID_ARG, "dictionary: missing '}'");
                return true;
            }
            if (k == 1) {
                if (t == "}") {
                    if (closed) return true;
                    return fail(FVGB_ERR_INVALID_ARG, "dictionary: unbalanced '}'");
                }
                if (t == ";") continue;
                return fail(FVGB_ERR_INVALID_ARG, "dictionary: unexpected '" + t + "' where a keyword belongs");
            }
            if (k == 2 && t[0] == '#') {
                if (!directive(lx, d, dir, t)) return false;
                continue;
            }
            if (k == 2 && t.size() > 1 && t[0] == '$') {  // $name; merges a sub-dictionary
                const std::string name = t.substr(1);
                const fvgb_dict::Entry* e = find_scoped(d, name);
                if (!e) return fail(FVGB_ERR_INVALID_ARG, "dictionary: undefined variable $" + name);
                if (!e->sub) return fail(FVGB_ERR_UNSUPPORTED, "dictionary: $" + name + " as an entry must name a sub-dictionary");
                const std::unique_ptr<fvgb_dict> copy = deep_copy(e->sub.get(), nullptr);
                merge_into(d, copy.get());
                const size_t p = lx.save();
                std::string semi;
                if (lx.next(semi) != 1 || semi != ";") lx.restore(p);
                continue;
            }
            fvgb_dict::Entry e;
            e.key = t;
            e.pattern = k == 3;
            const size_t p = lx.save();
            std::string nx;
            const int kk = lx.next(nx);
            if (kk == 1 && nx == "{") {
                e.sub = std::make_unique<fvgb_dict>();
                e.sub->parent = d;
                // merge into an existing sub-dictionary of the same keyword
                const int at = find_exact(d, e.key, e.pattern);
                if (at >= 0 && d->entries[at].sub) {
                    if (!body(lx, d->entries[at].sub.get(), dir, true)) return false;
                    continue;
                }
                if (!body(lx, e.sub.get(), dir, true)) return false;
                if (at >= 0) d->entries[at] = std::move(e);
                else d->entries.push_back(std::move(e));
                continue;
            }
            lx.restore(p);
            if (!read_value(lx, d, e.toks)) return false;
            put_entry(d, e);
        }
    }

    bool directive(Lex& lx, fvgb_dict* d, const std::string& dir, const std::string& name) {
        std::string t;
        if (name == "#include" || name == "#includeIfPresent" || name == "#sinclude") {
            const int k = lx.next(t);
            if (k != 3 && k != 2) return fail(FVGB_ERR_INVALID_ARG, "dictionary: " + name + " needs a file name");
            const std::string path = (!t.empty() && t[0] == '/') ? t : dir + "/" + t;
            return include(path, d, name != "#include");
        }
        if (name == "#inputMode") {
            lx.next(t);
            return true;
        }
        if (name == "#remove") {
            const int k = lx.next(t);
            std::vector<std::string> keys;
            if (k == 1 && t == "(") {
                while (lx.next(t) > 0 && t != ")") keys.push_back(t);
            } else if (k == 2 || k == 3) {
                keys.push_back(t);
            } else {
                return fail(FVGB_ERR_INVALID_ARG, "dictionary: #remove needs a keyword or a list");
            }
            for (const auto& key : keys) {
                const int at = find_entry(d, key);
                if (at >= 0) d->entries.erase(d->entries.begin() + at);
            }
            return true;
        }
        return fail(FVGB_ERR_UNSUPPORTED, "dictionary: directive " + name + " is not supported");
    }
};

fvgb_status parse_text(std::string text, const std::string& dir, fvgb_dict** out) {
    auto d = std::make_unique<fvgb_dict>();
    d->top = true;
    Parser ps;
    Lex lx;
    lx.s = std::move(text);
    if (!ps.body(lx, d.get(), dir, false)) return fvgb_fail((fvgb_status)ps.status, ps.err.c_str());
    const int h = find_exact(d.get(), "FoamFile", false);
    if (h >= 0 && d->entries[h].sub) d->entries.erase(d->entries.begin() + h);
    *out = d.release();
    return FVGB_OK;
}

// ------------------------------------------------ typed views used below
const fvgb_dict::Entry* entry_of(const fvgb_dict* d, const char* key) {
    const int i = find_entry(d, key);
    return i < 0 ? nullptr : &d->entries[i];
}

bool word_of(const fvgb_dict* d, const char* key, std::string& w) {
    const fvgb_dict::Entry* e = entry_of(d, key);
    if (!e || e->sub || e->toks.size() != 1) return false;
    const Tok& t = e->toks[0];
    if (t.kind != FVGB_TOK_WORD && t.kind != FVGB_TOK_STRING) return false;
    w = t.text;
    return true;
}

bool number_of(const fvgb_dict* d, const char* key, double& v) {
    const fvgb_dict::Entry* e = entry_of(d, key);
    if (!e || e->sub || e->toks.size() != 1) return false;
    const Tok& t = e->toks[0];
    if (t.kind != FVGB_TOK_LABEL && t.kind != FVGB_TOK_SCALAR) return false;
    v = t.scalar;
    return true;
}

void set_tokens(fvgb_dict* d, const std::string& key, std::vector<Tok> toks) {
    fvgb_dict::Entry e;
    e.key = key;
    e.toks = std::move(toks);
    const int at = find_exact(d, key, false);
    if (at >= 0) d->entries[at] = std::move(e);
    else d->entries.push_back(std::move(e));
}

void set_word(fvgb_dict* d, const std::string& key, const std::string& w, bool quoted) {
    Tok t;
    t.kind = quoted ? FVGB_TOK_STRING : FVGB_TOK_WORD;
    t.text = w;
    set_tokens(d, key, {t});
}

void set_number(fvgb_dict* d, const std::string& key, const Tok& num) { set_tokens(d, key, {num}); }

fvgb_dict* set_dict(fvgb_dict* d, const std::string& key) {
    fvgb_dict::Entry e;
    e.key = key;
    e.sub = std::make_unique<fvgb_dict>();
    e.sub->parent = d;
    fvgb_dict* s = e.sub.get();
    const int at = find_exact(d, key, false);
    if (at >= 0) d->entries[at] = std::move(e);
    else d->entries.push_back(std::move(e));
    return s;
}

void remove_key(fvgb_dict* d, const char* key) {
    const int at = find_entry(d, key);
    if (at >= 0) d->entries.erase(d->entries.begin() + at);
}

Tok label_tok(int64_t v) {
    Tok t;
    t.kind = FVGB_TOK_LABEL;
    t.label = v;
    t.scalar = (double)v;
    t.text = std::to_string(v);
    return t;
}

// ------------------------------------------------------------ writer
void write_tokens(std::ostringstream& o, const std::vector<Tok>& toks) {
    bool first = true;
    for (const Tok& t : toks) {
        if (!first && !(t.kind == FVGB_TOK_PUNCT && (t.text == ")" || t.text == "]"))) o << ' ';
        if (t.kind == FVGB_TOK_STRING) o << '"' << t.text << '"';
        else o << t.text;
        first = t.kind == FVGB_TOK_PUNCT && (t.text == "(" || t.text == "[");
    }
}

void write_dict(std::ostringstream& o, const fvgb_dict* d, int indent) {
    const std::string pad(indent * 4, ' ');
    for (const auto& e : d->entries) {
        o << pad;
        if (e.pattern) o << '"' << e.key << '"';
        else o << e.key;
        if (e.sub) {
            o << "\n" << pad << "{\n";
            write_dict(o, e.sub.get(), indent + 1);
            o << pad << "}\n";
        } else {
            o << ' ';
            write_tokens(o, e.toks);
            o << ";\n";
        }
    }
}

}  // namespace

// ====================================================================== C ABI
extern "C" fvgb_status fvgb_dict_read(const char* path, fvgb_dict** out) {
    if (!path || !out) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_read: null argument");
    *out = nullptr;
    std::string text;
    if (!read_file(path, text)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_read: cannot read the file");
    return parse_text(std::move(text), dir_of(path), out);
}

extern "C" fvgb_status fvgb_dict_parse(const char* text, const char* include_dir, fvgb_dict** out) {
    if (!text || !out) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_parse: null argument");
    *out = nullptr;
    return parse_text(text, include_dir ? include_dir : ".", out);
}

extern "C" fvgb_status fvgb_dict_create(fvgb_dict** out) {
    if (!out) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_create: null argument");
    auto d = std::make_unique<fvgb_dict>();
    d->top = true;
    *out = d.release();
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_dict_copy(const fvgb_dict* d, fvgb_dict** out) {
    if (!d || !out) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_copy: null argument");
    std::unique_ptr<fvgb_dict> c = deep_copy(d, nullptr);
    c->top = true;
    *out = c.release();
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_dict_free(fvgb_dict* d) {
    if (!d) return FVGB_OK;
    if (!d->top) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_free: not a top-level dictionary");
    delete d;
    return FVGB_OK;
}

extern "C" int32_t fvgb_dict_size(const fvgb_dict* d) { return d ? (int32_t)d->entries.size() : 0; }

extern "C" const char* fvgb_dict_key(const fvgb_dict* d, int32_t i) {
    if (!d || i < 0 || i >= (int32_t)d->entries.size()) return nullptr;
    return d->entries[i].key.c_str();
}

extern "C" int32_t fvgb_dict_is_pattern(const fvgb_dict* d, int32_t i) {
    if (!d || i < 0 || i >= (int32_t)d->entries.size()) return 0;
    return d->entries[i].pattern ? 1 : 0;
}

extern "C" int32_t fvgb_dict_find(const fvgb_dict* d, const char* keyword) {
    if (!d || !keyword) return -1;
    return find_entry(d, keyword);
}

extern "C" fvgb_dict* fvgb_dict_sub(const fvgb_dict* d, int32_t i) {
    if (!d || i < 0 || i >= (int32_t)d->entries.size()) return nullptr;
    return d->entries[i].sub.get();
}

extern "C" int32_t fvgb_dict_ntokens(const fvgb_dict* d, int32_t i) {
    if (!d || i < 0 || i >= (int32_t)d->entries.size() || d->entries[i].sub) return -1;
    return (int32_t)d->entries[i].toks.size();
}

extern "C" fvgb_status fvgb_dict_token(const fvgb_dict* d, int32_t i, int32_t j, int32_t* kind, const char** text,
                                       int64_t* label, double* scalar) {
    if (!d || i < 0 || i >= (int32_t)d->entries.size() || d->entries[i].sub)
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_token: no primitive entry at this index");
    const auto& toks = d->entries[i].toks;
    if (j < 0 || j >= (int32_t)toks.size()) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_token: token index");
    if (kind) *kind = toks[j].kind;
    if (text) *text = toks[j].text.c_str();
    if (label) *label = toks[j].label;
    if (scalar) *scalar = toks[j].scalar;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_dict_set(fvgb_dict* d, const char* keyword, const char* value) {
    if (!d || !keyword || !value) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_set: null argument");
    Parser ps;
    Lex lx;
    lx.s = std::string(value) + " ;";
    std::vector<Tok> toks;
    if (!ps.read_value(lx, d, toks)) return fvgb_fail((fvgb_status)ps.status, ps.err.c_str());
    std::string rest;
    if (lx.next(rest) != 0) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_set: ';' inside the value");
    set_tokens(d, keyword, std::move(toks));
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_dict_set_dict(fvgb_dict* d, const char* keyword, const fvgb_dict* src, fvgb_dict** sub) {
    if (!d || !keyword) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_set_dict: null argument");
    for (const fvgb_dict* a = d; a; a = a->parent)
        if (a == src) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_set_dict: a dictionary cannot contain itself");
    std::unique_ptr<fvgb_dict> copy = src ? deep_copy(src, nullptr) : nullptr;
    fvgb_dict* s = set_dict(d, keyword);
    if (copy) merge_into(s, copy.get());
    if (sub) *sub = s;
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_dict_remove(fvgb_dict* d, const char* keyword) {
    if (!d || !keyword) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_remove: null argument");
    remove_key(d, keyword);
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_dict_write(const fvgb_dict* d, char* buf, int64_t cap, int64_t* len) {
    if (!d) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_dict_write: null dictionary");
    std::ostringstream o;
    write_dict(o, d, 0);
    const std::string s = o.str();
    if (len) *len = (int64_t)s.size();
    if (buf && cap > 0) {
        const size_t n = std::min<size_t>(s.size(), (size_t)cap - 1);
        std::memcpy(buf, s.data(), n);
        buf[n] = '\0';
    }
    return FVGB_OK;
}

// ------------------------------------------------ fvSolution.cpp:19-159
extern "C" fvgb_status fvgb_fvsolution_update_solver(fvgb_dict* d) {
    if (!d) return fvgb_fail(FVGB_ERR_INVALID_ARG, "update_solver: null dictionary");
    static const char* kMap[][2] = {{"PCG", "solver::Cg"},
                                    {"PBiCG", "solver::Bicg"},
                                    {"PBiCGStab", "solver::Bicgstab"},
                                    {"smoothSolver", "solver::Bicgstab"},
                                    {"GAMG", "solver::Multigrid"}};
    std::string name;
    if (!word_of(d, "solver", name)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "update_solver: no 'solver' word");
    for (const auto& m : kMap) {
        if (name == m[0]) {
            set_word(d, "solver", "Ginkgo", false);
            set_word(d, "type", m[1], true);
            break;
        }
    }
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_fvsolution_update_preconditioner(fvgb_dict* d) {
    if (!d) return fvgb_fail(FVGB_ERR_INVALID_ARG, "update_preconditioner: null dictionary");
    auto put_mapped = [d](const std::string& name) {
        fvgb_dict* p = set_dict(d, "preconditioner");
        if (name == "DIC") {
            set_word(p, "type", "preconditioner::Jacobi", true);
            set_number(p, "max_block_size", label_tok(1));
        } else {  // DILU
            set_word(p, "type", "preconditioner::Ilu", true);
            set_word(p, "reverse_apply", "false", false);
            fvgb_dict* f = set_dict(p, "factorization");
            set_word(f, "type", "factorization::ParIlu", true);
        }
    };
    if (!entry_of(d, "preconditioner")) put_mapped("DIC");
    remove_key(d, "smoother");
    const fvgb_dict::Entry* e = entry_of(d, "preconditioner");
    if (e->sub) {
        const fvgb_dict::Entry* t = entry_of(e->sub.get(), "type");
        if (t && t->sub)
            return fvgb_fail(FVGB_ERR_UNSUPPORTED,
                             "GAMG is not supported in FoamAdapter, please use a different preconditioner.");
        return FVGB_OK;
    }
    std::string name;
    if (!word_of(d, "preconditioner", name)) return FVGB_OK;
    if (name == "DIC" || name == "DILU") put_mapped(name);
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_fvsolution_update_criteria(fvgb_dict* d) {
    if (!d) return fvgb_fail(FVGB_ERR_INVALID_ARG, "update_criteria: null dictionary");
    const fvgb_dict::Entry* ce = entry_of(d, "criteria");
    fvgb_dict* c = (ce && ce->sub) ? ce->sub.get() : set_dict(d, "criteria");
    set_number(c, "iteration", label_tok(1000));
    auto move_number = [&](const char* from, const char* to) -> bool {
        const fvgb_dict::Entry* e = entry_of(d, from);
        if (!e) return true;
        if (e->sub || e->toks.size() != 1 ||
            (e->toks[0].kind != FVGB_TOK_LABEL && e->toks[0].kind != FVGB_TOK_SCALAR))
            return false;
        set_number(c, to, e->toks[0]);
        remove_key(d, from);
        return true;
    };
    if (!move_number("relTol", "relative_residual_norm"))
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "update_criteria: relTol is not a number");
    if (!move_number("maxIter", "iteration"))
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "update_criteria: maxIter is not a number");
    if (!move_number("tolerance", "absolute_residual_norm"))
        return fvgb_fail(FVGB_ERR_INVALID_ARG, "update_criteria: tolerance is not a number");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_fvsolution_map(const fvgb_dict* solver_dict, fvgb_dict** mapped) {
    if (!solver_dict || !mapped) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_fvsolution_map: null argument");
    *mapped = nullptr;
    fvgb_dict* m = nullptr;
    fvgb_status st = fvgb_dict_copy(solver_dict, &m);
    if (st != FVGB_OK) return st;
    if (!entry_of(m, "configFile")) {
        if ((st = fvgb_fvsolution_update_solver(m)) != FVGB_OK ||
            (st = fvgb_fvsolution_update_preconditioner(m)) != FVGB_OK ||
            (st = fvgb_fvsolution_update_criteria(m)) != FVGB_OK) {
            fvgb_dict_free(m);
            return st;
        }
    }
    *mapped = m;
    return FVGB_OK;
}

// A preconditioner::Ilu entry this library implements: CG or BiCGStab,
// reverse_apply false (or absent), and a ParIlu (or exact Ilu) factorization,
// both of whose fixed points are the ILU(0) factors the library forms.
static fvgb_status ilu_entry_ok(const fvgb_dict* p, int32_t method) {
    if (method != FVGB_SOLVER_CG && method != FVGB_SOLVER_BICGSTAB)
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "solver entry: preconditioner::Ilu with Cg or Bicgstab only");
    std::string w;
    if (word_of(p, "reverse_apply", w) && w != "false")
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "solver entry: preconditioner::Ilu with reverse_apply true");
    const fvgb_dict::Entry* f = entry_of(p, "factorization");
    if (f && (!f->sub || !word_of(f->sub.get(), "type", w) ||
              (w != "factorization::ParIlu" && w != "factorization::Ilu")))
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "solver entry: ILU factorizations other than ParIlu / Ilu");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_solver_cfg_from_dict(const fvgb_dict* d, fvgb_solver_cfg* cfg) {
    if (!d || !cfg) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_solver_cfg_from_dict: null argument");
    fvgb_solver_cfg c{};
    c.max_iter = 1000;
    c.precision = FVGB_PREC_FP64;
    c.inner_rel_tol = 0.0;
    c.inner_max_iter = 1000;
    c.max_outer = 50;
    c.method = FVGB_SOLVER_CG;
    if (entry_of(d, "configFile"))
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "solver entry: configFile names a Ginkgo JSON file: fvgb_solver_cfg_from_json");
    std::string w;
    if (word_of(d, "solver", w) && w != "Ginkgo")
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, ("solver entry: solver " + w + " (map it with fvgb_fvsolution_map first)").c_str());
    if (!word_of(d, "type", w)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "solver entry: no Ginkgo solver type");
    if (w == "solver::Cg") c.method = FVGB_SOLVER_CG;
    else if (w == "solver::Bicgstab") c.method = FVGB_SOLVER_BICGSTAB;
    else if (w == "solver::Bicg") c.method = FVGB_SOLVER_BICG;
    else if (w == "solver::Multigrid") c.method = FVGB_SOLVER_MULTIGRID;
    else
        return fvgb_fail(FVGB_ERR_UNSUPPORTED,
                         ("solver entry: " + w + " is not implemented (Cg, Bicgstab, Bicg, Multigrid are)").c_str());
    const fvgb_dict::Entry* pe = entry_of(d, "preconditioner");
    const char* kPrecMsg =
        "solver entry: preconditioner::Jacobi with max_block_size 1 and solver::Multigrid (with CG) are implemented";
    double mbs = 0.0;
    if (c.method == FVGB_SOLVER_MULTIGRID) {
        // GAMG mapped (fvSolution.cpp:27): the multigrid solver; the Jacobi
        // preconditioner entry updatePreconditioner inserts is its smoother's
        if (pe && pe->sub &&
            (!word_of(pe->sub.get(), "type", w) || w != "preconditioner::Jacobi" ||
             !number_of(pe->sub.get(), "max_block_size", mbs) || mbs != 1.0))
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, "solver entry: solver::Multigrid smooths with Jacobi (block size 1) only");
    } else if (!pe || !pe->sub) {
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, kPrecMsg);
    } else if (word_of(pe->sub.get(), "type", w) && w == "solver::Multigrid" && c.method == FVGB_SOLVER_CG) {
        c.preconditioner = FVGB_PRECOND_MULTIGRID;
    } else if (word_of(pe->sub.get(), "type", w) && w == "preconditioner::Ilu") {
        // DILU mapped (fvSolution.cpp:56-63): ILU(0) with a ParIlu factorization, L applied first
        fvgb_status st = ilu_entry_ok(pe->sub.get(), c.method);
        if (st != FVGB_OK) return st;
        c.preconditioner = FVGB_PRECOND_ILU;
    } else if (!word_of(pe->sub.get(), "type", w) || w != "preconditioner::Jacobi" ||
               !number_of(pe->sub.get(), "max_block_size", mbs) || mbs != 1.0) {
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, kPrecMsg);
    }
    const fvgb_dict::Entry* ce = entry_of(d, "criteria");
    if (ce && ce->sub) {
        double v = 0.0;
        if (number_of(ce->sub.get(), "iteration", v)) c.max_iter = (int32_t)v;
        if (number_of(ce->sub.get(), "relative_residual_norm", v)) c.rel_tol = v;
        if (number_of(ce->sub.get(), "absolute_residual_norm", v)) c.abs_tol = v;
    }
    // extensions of this library (not FoamAdapter keywords)
    if (word_of(d, "precision", w)) {
        if (w == "mixed") c.precision = FVGB_PREC_MIXED_IR;
        else if (w != "FP64") return fvgb_fail(FVGB_ERR_INVALID_ARG, "solver entry: precision must be FP64 or mixed");
    }
    double v = 0.0;
    if (number_of(d, "innerRelTol", v)) c.inner_rel_tol = v;
    if (number_of(d, "innerMaxIter", v)) c.inner_max_iter = (int32_t)v;
    if (number_of(d, "maxOuter", v)) c.max_outer = (int32_t)v;
    if (c.inner_rel_tol <= 0.0) c.inner_rel_tol = c.method == FVGB_SOLVER_BICGSTAB ? 0.01 : 0.1;
    *cfg = c;
    return FVGB_OK;
}

// ------------------------------------------------- Ginkgo JSON configurations
// The configFile of a solver entry (fvSolution.cpp:145-152) is a Ginkgo JSON
// configuration, e.g. tutorials/cylinder2D/system/gko/config.mg.json.  A small
// JSON reader (objects, arrays, strings, numbers, true/false/null) and the
// mapping of the keys this library implements.
namespace {

using fvgb_json::Json;
using fvgb_json::JsonParser;

// a solver::Multigrid object's mg_level entries: multigrid::Pgm only
fvgb_status pgm_levels_only(const Json& mg) {
    const Json* lv = mg.get("mg_level");
    if (lv && lv->kind == Json::ARR)
        for (const Json& l : lv->arr) {
            const Json* lt = l.get("type");
            if (!lt || lt->kind != Json::STR || lt->str != "multigrid::Pgm")
                return fvgb_fail(FVGB_ERR_UNSUPPORTED, "Ginkgo config: multigrid levels other than multigrid::Pgm");
        }
    return FVGB_OK;
}

fvgb_status cfg_from_json(const Json& j, fvgb_solver_cfg* out) {
    fvgb_solver_cfg c{};
    c.max_iter = 1000;
    c.precision = FVGB_PREC_FP64;
    c.inner_max_iter = 1000;
    c.max_outer = 50;
    const Json* t = j.get("type");
    if (!t || t->kind != Json::STR) return fvgb_fail(FVGB_ERR_INVALID_ARG, "Ginkgo config: no solver type");
    if (t->str == "solver::Cg") c.method = FVGB_SOLVER_CG;
    else if (t->str == "solver::Bicgstab") c.method = FVGB_SOLVER_BICGSTAB;
    else if (t->str == "solver::Bicg") c.method = FVGB_SOLVER_BICG;
    else if (t->str == "solver::Multigrid") c.method = FVGB_SOLVER_MULTIGRID;
    else
        return fvgb_fail(FVGB_ERR_UNSUPPORTED,
                         ("Ginkgo config: " + t->str + " is not implemented (Cg, Bicgstab, Bicg, Multigrid are)").c_str());
    const Json* p = j.get("preconditioner");
    const Json* pt = p ? p->get("type") : nullptr;
    if (c.method == FVGB_SOLVER_MULTIGRID) {  // the solver itself: Pgm levels, no preconditioner
        fvgb_status ls = pgm_levels_only(j);
        if (ls != FVGB_OK) return ls;
        if (p) return fvgb_fail(FVGB_ERR_UNSUPPORTED, "Ginkgo config: solver::Multigrid takes no preconditioner");
    } else if (!pt || pt->kind != Json::STR) {
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, "Ginkgo config: an unpreconditioned solver is not implemented");
    } else if (pt->str == "preconditioner::Jacobi") {
        const Json* mbs = p->get("max_block_size");
        if (!mbs || mbs->kind != Json::NUM || mbs->num != 1.0)
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, "Ginkgo config: Jacobi with max_block_size 1 only");
    } else if (pt->str == "solver::Multigrid" && c.method == FVGB_SOLVER_CG) {
        fvgb_status ls = pgm_levels_only(*p);
        if (ls != FVGB_OK) return ls;
        c.preconditioner = FVGB_PRECOND_MULTIGRID;
    } else if (pt->str == "preconditioner::Ilu") {
        if (c.method != FVGB_SOLVER_CG && c.method != FVGB_SOLVER_BICGSTAB)
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, "Ginkgo config: preconditioner::Ilu with Cg or Bicgstab only");
        const Json* ra = p->get("reverse_apply");
        if (ra && !(ra->kind == Json::BOOL && !ra->b))
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, "Ginkgo config: preconditioner::Ilu with reverse_apply true");
        const Json* f = p->get("factorization");
        const Json* ft = f ? f->get("type") : nullptr;
        if (f && (!ft || ft->kind != Json::STR || (ft->str != "factorization::ParIlu" && ft->str != "factorization::Ilu")))
            return fvgb_fail(FVGB_ERR_UNSUPPORTED, "Ginkgo config: ILU factorizations other than ParIlu / Ilu");
        c.preconditioner = FVGB_PRECOND_ILU;
    } else {
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, ("Ginkgo config: preconditioner " + pt->str + " is not implemented").c_str());
    }
    const Json* cr = j.get("criteria");
    if (cr && cr->kind == Json::ARR) {
        for (const Json& k : cr->arr) {
            const Json* ct = k.get("type");
            if (!ct || ct->kind != Json::STR) return fvgb_fail(FVGB_ERR_INVALID_ARG, "Ginkgo config: criterion without type");
            if (ct->str == "Iteration") {
                const Json* m = k.get("max_iters");
                if (!m || m->kind != Json::NUM) return fvgb_fail(FVGB_ERR_INVALID_ARG, "Ginkgo config: Iteration without max_iters");
                c.max_iter = (int32_t)m->num;
            } else if (ct->str == "ResidualNorm") {
                const Json* f = k.get("reduction_factor");
                const Json* b = k.get("baseline");
                if (!f || f->kind != Json::NUM)
                    return fvgb_fail(FVGB_ERR_INVALID_ARG, "Ginkgo config: ResidualNorm without reduction_factor");
                const std::string base = (b && b->kind == Json::STR) ? b->str : "rhs_norm";
                if (base == "absolute") {
                    c.abs_tol = f->num;
                } else if (base == "initial_resnorm") {
                    c.rel_tol = f->num;
                } else if (base == "rhs_norm") {  // Ginkgo's default: ||r|| <= f ||b||
                    c.rel_tol = f->num;
                    c.flags |= FVGB_SOLVE_RHS_BASELINE;
                } else {
                    return fvgb_fail(FVGB_ERR_INVALID_ARG, ("Ginkgo config: ResidualNorm baseline " + base +
                                                            " is not one of rhs_norm, initial_resnorm, absolute").c_str());
                }
            } else {
                return fvgb_fail(FVGB_ERR_UNSUPPORTED, ("Ginkgo config: criterion " + ct->str + " is not implemented").c_str());
            }
        }
    }
    c.inner_rel_tol = c.method == FVGB_SOLVER_BICGSTAB ? 0.01 : 0.1;
    *out = c;
    return FVGB_OK;
}

}  // namespace

extern "C" fvgb_status fvgb_solver_cfg_from_json(const char* path, fvgb_solver_cfg* cfg) {
    if (!path || !cfg) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_solver_cfg_from_json: null argument");
    std::string text;
    if (!read_file(path, text)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_solver_cfg_from_json: cannot read the file");
    Json j;
    JsonParser ps(text);
    if (!ps.value(j) || j.kind != Json::OBJ) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_solver_cfg_from_json: malformed JSON");
    ps.ws();
    if (ps.i != text.size()) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_solver_cfg_from_json: text after the JSON object");
    return cfg_from_json(j, cfg);
}

// ------------------------------------------------------------ fvSchemes
extern "C" fvgb_status fvgb_scheme_from_dict(const fvgb_dict* schemes, const char* section, const char* name,
                                             int32_t* scheme) {
    if (!schemes || !section || !name || !scheme) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_scheme_from_dict: null argument");
    const fvgb_dict::Entry* se = entry_of(schemes, section);
    if (!se || !se->sub) return fvgb_fail(FVGB_ERR_INVALID_ARG, (std::string("fvSchemes: no ") + section).c_str());
    const fvgb_dict* s = se->sub.get();
    const fvgb_dict::Entry* e = entry_of(s, name);
    if (!e) e = entry_of(s, "default");
    if (!e || e->sub || e->toks.empty() || e->toks[0].text == "none")
        return fvgb_fail(FVGB_ERR_INVALID_ARG, (std::string("fvSchemes: no scheme for ") + name + " in " + section).c_str());
    std::vector<std::string> w;
    for (const Tok& t : e->toks) w.push_back(t.text);
    const std::string sec = section;
    auto is = [&w](std::initializer_list<const char*> want) {
        if (w.size() != want.size()) return false;
        size_t k = 0;
        for (const char* x : want)
            if (w[k++] != x) return false;
        return true;
    };
    int32_t r = -1;
    if (sec == "divSchemes" || sec == "gradSchemes") {
        if (is({"Gauss", "linear"})) r = FVGB_SCHEME_LINEAR;
        else if (sec == "divSchemes" && is({"Gauss", "upwind"})) r = FVGB_SCHEME_UPWIND;
    } else if (sec == "laplacianSchemes") {
        if (is({"Gauss", "linear", "uncorrected"})) r = 0;
        else if (is({"Gauss", "linear", "corrected"})) r = FVGB_SCHEME_CORRECTED;
    } else if (sec == "snGradSchemes") {
        if (is({"uncorrected"})) r = 0;
        else if (is({"corrected"})) r = FVGB_SCHEME_CORRECTED;
    } else if (sec == "interpolationSchemes") {
        if (is({"linear"})) r = FVGB_SCHEME_LINEAR;
        else if (!w.empty() && w[0] == "upwind") r = FVGB_SCHEME_UPWIND;
    } else if (sec == "ddtSchemes") {
        if (is({"Euler"})) r = 0;
    } else {
        return fvgb_fail(FVGB_ERR_INVALID_ARG, ("fvSchemes: unknown section " + sec).c_str());
    }
    if (r < 0) {
        std::string all;
        for (const auto& x : w) all += (all.empty() ? "" : " ") + x;
        return fvgb_fail(FVGB_ERR_UNSUPPORTED, ("fvSchemes: " + sec + " " + name + ": '" + all + "' is not implemented").c_str());
    }
    *scheme = r;
    return FVGB_OK;
}
