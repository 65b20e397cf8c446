// lla_autotune.cpp -- see lla_autotune.h.
#include "lla_autotune.h"

#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <utility>

namespace lla {

namespace {

std::mutex g_mu;
std::string g_loaded_path;              // the file the map was read from
std::map<std::string, std::pair<int, int>> g_map;
bool g_loaded = false;

std::string cache_path() {
    const char *p = std::getenv("LLA_AUTOTUNE_CACHE");
    if (p && *p) return p;
    const char *h = std::getenv("HOME");
    return std::string(h ? h : "/tmp") + "/.cache/lla_gb300_autotune.txt";
}

// With g_mu held: the map reflects the current path's file.
void load(const std::string &path) {
    if (g_loaded && path == g_loaded_path) return;
    g_map.clear();
    g_loaded_path = path;
    g_loaded = true;
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char k[512];
    int a, b;
    while (std::fscanf(f, "%511s %d %d", k, &a, &b) == 3) g_map[k] = std::make_pair(a, b);
    std::fclose(f);
}

}  // namespace

bool autotune_lookup(const std::string &key, int &a, int &b) {
    std::lock_guard<std::mutex> lk(g_mu);
    load(cache_path());
    auto it = g_map.find(key);
    if (it == g_map.end()) return false;
    a = it->second.first;
    b = it->second.second;
    return true;
}

void autotune_store(const std::string &key, int a, int b) {
    std::lock_guard<std::mutex> lk(g_mu);
    const std::string path = cache_path();
    load(path);
    g_map[key] = std::make_pair(a, b);
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) {
        const std::string dir = path.substr(0, slash);
        for (size_t i = 1; i <= dir.size(); ++i)
            if (i == dir.size() || dir[i] == '/') (void)mkdir(dir.substr(0, i).c_str(), 0755);
    }
    FILE *f = std::fopen(path.c_str(), "a");
    if (!f) return;
    std::fprintf(f, "%s %d %d\n", key.c_str(), a, b);
    std::fclose(f);
}

}  // namespace lla
