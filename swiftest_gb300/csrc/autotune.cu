// autotune.cu -- persistent cache of the kernel-shape choices made by the autotuner.
//
// The batched mixed kick has several tile shapes that give identical results (see
// k_kick_mixed_batched); the ensemble times them on its own data the first time a
// (GPU, kick kind, radius guard, system-size bucket) combination is met and keeps the
// fastest.  Choices are kept for the process and appended to a small text file so later
// runs skip the timing: $SWG_TUNE_CACHE if set, else $HOME/.cache/swiftest_gb300/kick_tune.txt
// (no file is written when neither is available).  One line per choice: "<key> <variant>".
// The symmetric pl-pl kick's strip length is kept the same way, as log2(strip).
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>

#include "swg_internal.cuh"

namespace swg {

namespace {

std::mutex g_tune_mutex;
std::map<std::string, int> g_tune;
bool g_tune_loaded = false;

std::string cache_path() {
    if (const char *p = std::getenv("SWG_TUNE_CACHE")) return p;
    const char *home = std::getenv("HOME");
    if (!home || !*home) return "";
    const std::string dir = std::string(home) + "/.cache/swiftest_gb300";
    mkdir((std::string(home) + "/.cache").c_str(), 0755);
    mkdir(dir.c_str(), 0755);
    return dir + "/kick_tune.txt";
}

void load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const std::string path = cache_path();
    if (path.empty()) return;
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) return;
    char key[512];
    int v = 0;
    while (std::fscanf(f, "%511s %d", key, &v) == 2)
        if (v >= 0 && v < 16) g_tune[key] = v;  // callers check the range of their own keys
    std::fclose(f);
}

}  // namespace

std::string tune_key(int device, const char *kind, int bucket) {
    cudaDeviceProp prop;
    std::string name = "gpu";
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) name = prop.name;
    for (char &ch : name)
        if (ch == ' ' || ch == '|') ch = '_';
    return name + "|" + kind + "|b" + std::to_string(bucket);
}

int tune_lookup(const std::string &key) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    load_locked();
    auto it = g_tune.find(key);
    return it == g_tune.end() ? -1 : it->second;
}

void tune_store(const std::string &key, int variant) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    load_locked();
    g_tune[key] = variant;
    const std::string path = cache_path();
    if (path.empty()) return;
    if (FILE *f = std::fopen(path.c_str(), "a")) {
        std::fprintf(f, "%s %d\n", key.c_str(), variant);
        std::fclose(f);
    }
}

}  // namespace swg
