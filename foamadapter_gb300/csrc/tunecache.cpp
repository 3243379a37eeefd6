// The autotuner's cache: the kernel variants measured on a system, keyed by
// the system's shape (rows, slots per row, column-offset width, GPU), kept for
// the process and optionally in a JSON file, so that a later system of the same
// shape -- in this run or another, or a served request that may not be timed --
// starts with the measured choice instead of timing again.
//
// File format (written and read by this library):
//   {"version": 1, "entries": [
//     {"key": "...", "variants": [v_fp64_spmv, v_fp64_update, v_fp32_spmv, v_fp32_update],
//      "ms": [[...4 per kind...], ...]}, ...]}
// A variant of -1 means "not measured".  FVGB_TUNING_CACHE (environment)
// names a file that is read at the first lookup and rewritten whenever a new
// measurement is recorded.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>

#include "fvgb.h"
#include "fvgb_host_common.h"
#include "json_min.h"
#include "tunecache.h"

namespace {

struct Entry {
    int variant[kTuneCacheKinds] = {-1, -1, -1, -1};
    float ms[kTuneCacheKinds][kTuneCacheVariants] = {};
};

std::mutex g_mu;
std::map<std::string, Entry> g_entries;
bool g_env_read = false;
std::string g_autosave;

bool read_text(const char* path, std::string& out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

// merge the entries of a file; false (and nothing merged) on a malformed file
bool load_locked(const char* path, std::string* err) {
    std::string text;
    if (!read_text(path, text)) {
        *err = "cannot read the file";
        return false;
    }
    fvgb_json::Json j;
    fvgb_json::JsonParser ps(text);
    if (!ps.value(j) || j.kind != fvgb_json::Json::OBJ) {
        *err = "malformed JSON";
        return false;
    }
    const fvgb_json::Json* v = j.get("version");
    const fvgb_json::Json* es = j.get("entries");
    if (!v || v->kind != fvgb_json::Json::NUM || v->num != 1.0 || !es || es->kind != fvgb_json::Json::ARR) {
        *err = "not a version-1 tuning cache";
        return false;
    }
    std::map<std::string, Entry> add;
    for (const fvgb_json::Json& e : es->arr) {
        const fvgb_json::Json* k = e.get("key");
        const fvgb_json::Json* vs = e.get("variants");
        if (!k || k->kind != fvgb_json::Json::STR || !vs || vs->kind != fvgb_json::Json::ARR ||
            vs->arr.size() != (size_t)kTuneCacheKinds) {
            *err = "entry without key or four variants";
            return false;
        }
        for (char ch : k->str)
            if ((unsigned char)ch < 0x20) {
                *err = "key with a control character";
                return false;
            }
        Entry en;
        for (int q = 0; q < kTuneCacheKinds; ++q) {
            const fvgb_json::Json& x = vs->arr[q];
            if (x.kind != fvgb_json::Json::NUM || x.num < -1 || x.num >= kTuneCacheVariants || x.num != (int)x.num) {
                *err = "variant out of range";
                return false;
            }
            en.variant[q] = (int)x.num;
        }
        const fvgb_json::Json* ms = e.get("ms");
        if (ms && ms->kind == fvgb_json::Json::ARR && ms->arr.size() == (size_t)kTuneCacheKinds)
            for (int q = 0; q < kTuneCacheKinds; ++q)
                if (ms->arr[q].kind == fvgb_json::Json::ARR && ms->arr[q].arr.size() == (size_t)kTuneCacheVariants)
                    for (int w = 0; w < kTuneCacheVariants; ++w)
                        if (ms->arr[q].arr[w].kind == fvgb_json::Json::NUM) en.ms[q][w] = (float)ms->arr[q].arr[w].num;
        add[k->str] = en;
    }
    for (auto& kv : add) g_entries[kv.first] = kv.second;
    return true;
}

// a key as a JSON string body: quotes and backslashes escaped (keys hold no
// control characters: the library makes none and a load refuses them)
std::string json_escaped(const std::string& k) {
    std::string o;
    for (char ch : k) {
        if (ch == '"' || ch == '\\') o.push_back('\\');
        o.push_back(ch);
    }
    return o;
}

bool save_locked(const char* path) {
    std::ostringstream o;
    o << "{\"version\": 1, \"entries\": [";
    bool first = true;
    for (const auto& kv : g_entries) {
        o << (first ? "\n" : ",\n") << "  {\"key\": \"" << json_escaped(kv.first) << "\", \"variants\": [";
        for (int q = 0; q < kTuneCacheKinds; ++q) o << (q ? ", " : "") << kv.second.variant[q];
        o << "], \"ms\": [";
        for (int q = 0; q < kTuneCacheKinds; ++q) {
            o << (q ? ", [" : "[");
            for (int w = 0; w < kTuneCacheVariants; ++w) {
                char buf[32];
                std::snprintf(buf, sizeof buf, "%.6g", (double)kv.second.ms[q][w]);
                o << (w ? ", " : "") << buf;
            }
            o << "]";
        }
        o << "]}";
        first = false;
    }
    o << "\n]}\n";
    const std::string tmp = std::string(path) + ".tmp";
    {
        std::ofstream f(tmp, std::ios::binary | std::ios::trunc);
        if (!f) return false;
        f << o.str();
        if (!f) return false;
    }
    return std::rename(tmp.c_str(), path) == 0;
}

void read_env_locked() {
    if (g_env_read) return;
    g_env_read = true;
    const char* p = std::getenv("FVGB_TUNING_CACHE");
    if (!p || !*p) return;
    g_autosave = p;
    std::string err;
    load_locked(p, &err);  // a missing or unreadable file starts an empty cache
}

}  // namespace

bool tune_cache_get(const std::string& key, int kind, int* variant) {
    std::lock_guard<std::mutex> lk(g_mu);
    read_env_locked();
    auto it = g_entries.find(key);
    if (it == g_entries.end() || it->second.variant[kind] < 0) return false;
    *variant = it->second.variant[kind];
    return true;
}

void tune_cache_put(const std::string& key, int kind, int variant, const float* ms) {
    std::lock_guard<std::mutex> lk(g_mu);
    read_env_locked();
    Entry& e = g_entries[key];
    e.variant[kind] = variant;
    for (int w = 0; w < kTuneCacheVariants; ++w) e.ms[kind][w] = ms[w];
    if (!g_autosave.empty()) save_locked(g_autosave.c_str());
}

extern "C" fvgb_status fvgb_tuning_cache_load(const char* path) {
    fvgb_clear_error();
    if (!path) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_tuning_cache_load: null path");
    std::lock_guard<std::mutex> lk(g_mu);
    read_env_locked();
    std::string err;
    if (!load_locked(path, &err)) return fvgb_fail(FVGB_ERR_INVALID_ARG, ("fvgb_tuning_cache_load: " + err).c_str());
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_tuning_cache_save(const char* path) {
    fvgb_clear_error();
    if (!path) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_tuning_cache_save: null path");
    std::lock_guard<std::mutex> lk(g_mu);
    read_env_locked();
    if (!save_locked(path)) return fvgb_fail(FVGB_ERR_INVALID_ARG, "fvgb_tuning_cache_save: cannot write the file");
    return FVGB_OK;
}

extern "C" fvgb_status fvgb_tuning_cache_clear(void) {
    fvgb_clear_error();
    std::lock_guard<std::mutex> lk(g_mu);
    g_env_read = true;  // a cleared cache does not read the environment's file again
    g_entries.clear();
    return FVGB_OK;
}

extern "C" int32_t fvgb_tuning_cache_size(void) {
    std::lock_guard<std::mutex> lk(g_mu);
    read_env_locked();
    return (int32_t)g_entries.size();
}
