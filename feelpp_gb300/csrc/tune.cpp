// Launch-shape autotuner store.
//
// Kernels whose launch shape (threads per block, blocks per SM, contributions
// loaded per batch) does not change their results are timed on their real inputs
// the first time a (device, kernel, order, precision, size class) key is met,
// the fastest shape is kept and, when fgpu_config.tune_cache names a file,
// appended to it so that later processes start from it. The file holds one line
// per key: the key, then the integer parameters. Picks are kept per cache file
// (contexts without a file share one set), so a context given a new file tunes
// afresh.
#include <cstdio>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "fgpu_core.h"

namespace fgpu {

namespace {
std::mutex g_mutex;
std::map<std::string, std::map<std::string, std::vector<int>>> g_store;   // per cache file
}  // namespace

void tune_load_cache_file(const std::string& path) {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (path.empty()) return;
    auto& store = g_store[path];
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string key;
        if (!(ls >> key)) continue;
        std::vector<int> vals;
        int v;
        while (ls >> v) vals.push_back(v);
        if (!vals.empty()) store[key] = vals;         // a later line overrides an earlier one
    }
}

bool tune_lookup(const std::string& file, const std::string& key, std::vector<int>& vals) {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto& store = g_store[file];
    auto it = store.find(key);
    if (it == store.end()) return false;
    vals = it->second;
    return true;
}

void tune_record(const std::string& file, const std::string& key, const std::vector<int>& vals) {
    std::lock_guard<std::mutex> lock(g_mutex);
    g_store[file][key] = vals;
    if (file.empty()) return;
    std::ofstream out(file, std::ios::app);
    out << key;
    for (int v : vals) out << ' ' << v;
    out << '\n';
}

// key prefix: the device's name without blanks and its SM count
std::string tune_device_key(int device) {
    cudaDeviceProp p{};
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) {
        cudaGetLastError();
        return "device" + std::to_string(device);
    }
    std::string name = p.name;
    for (char& c : name)
        if (c == ' ' || c == '|') c = '_';
    return name + "-" + std::to_string(p.multiProcessorCount) + "sm";
}

// size class of a problem: floor(log2(n)) (n >= 1)
int tune_size_class(int64_t n) {
    int c = 0;
    while (n > 1) {
        n >>= 1;
        ++c;
    }
    return c;
}

}  // namespace fgpu
