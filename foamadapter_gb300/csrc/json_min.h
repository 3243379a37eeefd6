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
    bool string(std::string& out) {
        if (i >= s.size() || s[i] != '"') return false;
        ++i;
        out.clear();
        while (i < s.size() && s[i] != '"') {
            if (s[i] == '\\' && i + 1 < s.size()) {
                ++i;
                const char e = s[i];
                out.push_back(e == 'n' ? '\n' : e == 't' ? '\t' : e);
            } else {
                out.push_back(s[i]);
            }
            ++i;
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
