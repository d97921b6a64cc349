/*
 * Launch-policy knobs and the per-GPU tuning table.
 *
 * Every choice the library makes per size class (CTAs per network, kernel
 * variant, tile size, thresholds between kernels, threads per CTA,
 * escalation) reads a named knob.  A knob's value comes from, in order:
 *   1. the environment variable of that name (an explicit override);
 *   2. the tuning table loaded for the process: nr_tuning_load(path), else
 *      the file NR_TUNING_FILE names, else tuning/<device name>.txt beside
 *      libnetrelax.so (device name lowercased, other characters '_', e.g.
 *      tuning/nvidia_gb300.txt), which the autotuner
 *      (network_relaxation_gb300/autotune.py) writes from measurements on
 *      that GPU;
 *   3. the built-in default of the policy that asks.
 * Table lines are "NAME value" (NAME as the environment variable); '#'
 * starts a comment.
 */
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "nr_internal.h"

namespace nr {
namespace {

/* Every table and source name ever loaded stays allocated for the life of
 * the process: knob() and nr_tuning_source() hand out pointers into them,
 * which a later nr_tuning_load on another thread must not invalidate. */
using Table = std::map<std::string, std::string>;
std::mutex g_mu;
std::vector<std::unique_ptr<Table>> g_tables;
std::vector<std::unique_ptr<std::string>> g_sources;
const Table *g_table = nullptr;
const std::string *g_source = nullptr;
bool g_loaded = false;

void install_locked(Table &&t, const std::string &source) {
    g_tables.push_back(std::unique_ptr<Table>(new Table(std::move(t))));
    g_sources.push_back(std::unique_ptr<std::string>(new std::string(source)));
    g_table = g_tables.back().get();
    g_source = g_sources.back().get();
}

int parse_table(const std::string &path, std::map<std::string, std::string> &out) {
    std::ifstream in(path);
    if (!in.is_open()) return NR_ERR_IO;
    std::string line;
    int n = 0;
    while (std::getline(in, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        std::istringstream ss(line);
        std::string key, value, extra;
        if (!(ss >> key)) continue;
        if (!(ss >> value) || (ss >> extra)) return NR_ERR_PARSE;
        for (char c : key)
            if (!(isupper((unsigned char)c) || isdigit((unsigned char)c) || c == '_')) return NR_ERR_PARSE;
        out[key] = value;
        ++n;
    }
    return n;
}

/* tuning/<device name>.txt beside the library, for the current device. */
std::string default_table_path() {
    Dl_info info;
    if (!dladdr((const void *)&default_table_path, &info) || !info.dli_fname) return "";
    std::string dir = info.dli_fname;
    const size_t slash = dir.rfind('/');
    dir = slash == std::string::npos ? std::string(".") : dir.substr(0, slash);
    int dev = 0;
    cudaDeviceProp prop;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        return "";
    }
    std::string name;
    for (const char *c = prop.name; *c; ++c) name += isalnum((unsigned char)*c) ? (char)tolower((unsigned char)*c) : '_';
    return dir + "/tuning/" + name + ".txt";
}

void load_default_locked() {
    if (g_loaded) return;
    g_loaded = true;
    const char *env = getenv("NR_TUNING_FILE");
    const std::string path = env ? std::string(env) : default_table_path();
    if (path.empty()) return;
    Table t;
    if (parse_table(path, t) >= 0) install_locked(std::move(t), path);
}

}  // namespace

const char *knob(const char *name) {
    const char *env = getenv(name);
    if (env) return env;
    std::lock_guard<std::mutex> lock(g_mu);
    load_default_locked();
    if (!g_table) return nullptr;
    auto it = g_table->find(name);
    return it == g_table->end() ? nullptr : it->second.c_str();
}

}  // namespace nr

using namespace nr;

extern "C" {

int nr_tuning_load(const char *path) {
    if (!path) return fail(NR_ERR_INVALID, "nr_tuning_load: null path");
    Table t;
    const int n = parse_table(path, t);
    if (n == NR_ERR_IO) return fail(NR_ERR_IO, std::string("cannot open ") + path);
    if (n < 0) return fail(NR_ERR_PARSE, std::string("malformed tuning table ") + path);
    std::lock_guard<std::mutex> lock(g_mu);
    install_locked(std::move(t), path);
    g_loaded = true;
    return n;
}

double nr_tuning_value(const char *name) {
    if (!name) return NAN;
    const char *v = knob(name);
    if (!v) return NAN;
    char *end = nullptr;
    const double x = strtod(v, &end);
    return end && end != v ? x : NAN;
}

const char *nr_tuning_source(void) {
    std::lock_guard<std::mutex> lock(g_mu);
    load_default_locked();
    return g_source ? g_source->c_str() : "";
}

}  // extern "C"
