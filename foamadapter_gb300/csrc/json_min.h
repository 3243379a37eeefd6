// A small JSON reader for the host code of libfvgb: objects, arrays, strings,
// numbers, true/false/null, nesting depth at most 64.  Used for Ginkgo
// solver configurations (foamdict.cpp) and the autotuner's cache file
// (tunecache.cpp).
#pragma once
#include <cctype>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

namespace fvgb_json {

struct Json {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;
    const Json* get(const char* k) const {
        for (const auto& kv : obj)
            if (kv.first == k) return &kv.second;
        return nullptr;
    }
};

struct JsonParser {
    const std::string& s;
    size_t i = 0;
    int depth = 0;
    explicit JsonParser(const std::string& t) : s(t) {}
    void ws() {
        while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    }
    bool lit(const char* w) {
        const size_t n = std::strlen(w);
        if (s.compare(i, n, w) != 0) return false;
        i += n;
        return true;
    }
    // four hex digits at s[at..at+4)
    bool hex4(size_t at, unsigned& u) const {
        if (at + 4 > s.size()) return false;
        u = 0;
        for (size_t k = at; k < at + 4; ++k) {
            const char c = s[k];
            const unsigned d = c >= '0' && c <= '9' ? (unsigned)(c - '0')
                               : c >= 'a' && c <= 'f' ? (unsigned)(c - 'a' + 10)
                               : c >= 'A' && c <= 'F' ? (unsigned)(c - 'A' + 10)
                                                      : 16u;
            if (d > 15) return false;
            u = u * 16 + d;
        }
        return true;
    }
    static void utf8(unsigned cp, std::string& out) {
        if (cp < 0x80) {
            out.push_back((char)cp);
        } else if (cp < 0x800) {
            out.push_back((char)(0xC0 | (cp >> 6)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        } else if (cp < 0x10000) {
            out.push_back((char)(0xE0 | (cp >> 12)));
            out.push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        } else {
            out.push_back((char)(0xF0 | (cp >> 18)));
            out.push_back((char)(0x80 | ((cp >> 12) & 0x3F)));
            out.push_back((char)(0x80 | ((cp >> 6) & 0x3F)));
            out.push_back((char)(0x80 | (cp & 0x3F)));
        }
    }
    // a JSON string with its escapes (\" \\ \/ \b \f \n \r \t \uXXXX, surrogate
    // pairs joined), as UTF-8
    bool string(std::string& out) {
        if (i >= s.size() || s[i] != '"') return false;
        ++i;
        out.clear();
        while (i < s.size() && s[i] != '"') {
            if (s[i] != '\\') {
                out.push_back(s[i++]);
                continue;
            }
            if (++i >= s.size()) return false;
            const char e = s[i++];
            switch (e) {
                case '"': case '\\': case '/': out.push_back(e); break;
                case 'b': out.push_back('\b'); break;
                case 'f': out.push_back('\f'); break;
                case 'n': out.push_back('\n'); break;
                case 'r': out.push_back('\r'); break;
                case 't': out.push_back('\t'); break;
                case 'u': {
                    unsigned cp;
                    if (!hex4(i, cp)) return false;
                    i += 4;
                    if (cp >= 0xD800 && cp < 0xDC00) {  // high surrogate: a low one must follow
                        unsigned lo;
                        if (i + 6 > s.size() || s[i] != '\\' || s[i + 1] != 'u' || !hex4(i + 2, lo) || lo < 0xDC00 ||
                            lo >= 0xE000)
                            return false;
                        i += 6;
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    } else if (cp >= 0xDC00 && cp < 0xE000) {
                        return false;
                    }
                    utf8(cp, out);
                    break;
                }
                default: return false;
            }
        }
        if (i >= s.size()) return false;
        ++i;
        return true;
    }
    bool value(Json& v) {
        if (++depth > 64) return false;
        ws();
        bool ok = false;
        if (i >= s.size()) {
            ok = false;
        } else if (s[i] == '{') {
            v.kind = Json::OBJ;
            ++i;
            ws();
            if (i < s.size() && s[i] == '}') {
                ++i;
                ok = true;
            } else {
                for (;;) {
                    ws();
                    std::string k;
                    Json x;
                    if (!string(k)) break;
                    ws();
                    if (i >= s.size() || s[i] != ':') break;
                    ++i;
                    if (!value(x)) break;
                    v.obj.emplace_back(k, std::move(x));
                    ws();
                    if (i < s.size() && s[i] == ',') {
                        ++i;
                        continue;
                    }
                    if (i < s.size() && s[i] == '}') {
                        ++i;
                        ok = true;
                    }
                    break;
                }
            }
        } else if (s[i] == '[') {
            v.kind = Json::ARR;
            ++i;
            ws();
            if (i < s.size() && s[i] == ']') {
                ++i;
                ok = true;
            } else {
                for (;;) {
                    Json x;
                    if (!value(x)) break;
                    v.arr.push_back(std::move(x));
                    ws();
                    if (i < s.size() && s[i] == ',') {
                        ++i;
                        continue;
                    }
                    if (i < s.size() && s[i] == ']') {
                        ++i;
                        ok = true;
                    }
                    break;
                }
            }
        } else if (s[i] == '"') {
            v.kind = Json::STR;
            ok = string(v.str);
        } else if (lit("true")) {
            v.kind = Json::BOOL;
            v.b = ok = true;
        } else if (lit("false")) {
            v.kind = Json::BOOL;
            ok = true;
        } else if (lit("null")) {
            ok = true;
        } else {
            const char* b0 = s.c_str() + i;
            char* end = nullptr;
            v.num = std::strtod(b0, &end);
            if (end != b0) {
                v.kind = Json::NUM;
                i += (size_t)(end - b0);
                ok = true;
            }
        }
        --depth;
        return ok;
    }
};

}  // namespace fvgb_json
