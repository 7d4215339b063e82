// Process-wide table of tuned launch parameters (tuner.h).
#include "tuner.h"

#include <atomic>
#include <cstdio>
#include <map>
#include <mutex>

namespace nvpt {
namespace tune {
namespace {
std::atomic<bool> g_on{false};
std::mutex g_mu;
struct Entry {
    int choice;
    std::string trials;
};
std::map<std::string, Entry> g_table;  // key = "dev<d>/<parameter>/<shape>"

std::string full_key(const std::string &key) {
    int dev = 0;
    cudaGetDevice(&dev);
    return "dev" + std::to_string(dev) + "/" + key;
}
}  // namespace

bool enabled() { return g_on.load(std::memory_order_relaxed); }
void set_enabled(bool on) { g_on.store(on, std::memory_order_relaxed); }

int lookup(const std::string &key) {
    std::lock_guard<std::mutex> g(g_mu);
    auto it = g_table.find(full_key(key));
    return it == g_table.end() ? -1 : it->second.choice;
}

void record(const std::string &key, int choice, const float *ms, const int *cand, int ncand) {
    std::string t;
    for (int i = 0; i < ncand; ++i) {
        char b[64];
        snprintf(b, sizeof b, "%s\"%d\": %.4f", i ? ", " : "", cand[i], ms[i]);
        t += b;
    }
    std::lock_guard<std::mutex> g(g_mu);
    g_table[full_key(key)] = Entry{choice, t};
}

std::string report() {
    std::lock_guard<std::mutex> g(g_mu);
    std::string s = "{";
    bool first = true;
    for (auto &kv : g_table) {
        s += (first ? "\"" : ", \"") + kv.first + "\": {\"choice\": " + std::to_string(kv.second.choice) +
             ", \"ms\": {" + kv.second.trials + "}}";
        first = false;
    }
    return s + "}";
}

void clear() {
    std::lock_guard<std::mutex> g(g_mu);
    g_table.clear();
}

}  // namespace tune
}  // namespace nvpt
