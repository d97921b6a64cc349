/*
 * Host-side network handling: the triple finder (get_triples), fcodes,
 * per-node incidence lists and the error plumbing of the C ABI (the .dat
 * reader and writer are in fast_io.cpp).
 *
 * Compiled with -ffp-contract=off: rest lengths and the triple test must
 * round exactly as the reference's host code (large_strain_relax.cu:97-99,
 * :157-168), which the host compiler builds without fused multiply-adds.
 */
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <thread>

#include "nr_internal.h"

namespace nr {

static thread_local std::string g_last_error;

int fail(int status, const std::string &msg) {
    g_last_error = msg;
    return status;
}
void clear_error() { g_last_error.clear(); }

void y_range(const std::vector<double> &points, double &miny, double &maxy) {
    miny = FLT_MAX;
    maxy = FLT_MIN;
    for (size_t i = 1; i < points.size(); i += 2) {
        const double y = points[i];
        if (y < miny) miny = y;
        if (y > maxy) maxy = y;
    }
}

void build_incidence(int n, const int *edge_ij, int n_edges, const int *tri_hjk, int n_triples, bool use_bonds,
                     bool use_triples, Incidence &inc) {
    inc.bptr.assign((size_t)n + 1, 0);
    inc.tptr.assign((size_t)n + 1, 0);
    if (use_bonds)
        for (int b = 0; b < n_edges; ++b) {
            inc.bptr[edge_ij[2 * b] + 1]++;
            inc.bptr[edge_ij[2 * b + 1] + 1]++;
        }
    if (use_triples)
        for (int t = 0; t < n_triples; ++t)
            for (int r = 0; r < 3; ++r) inc.tptr[tri_hjk[3 * t + r] + 1]++;
    for (int i = 0; i < n; ++i) {
        inc.bptr[i + 1] += inc.bptr[i];
        inc.tptr[i + 1] += inc.tptr[i];
    }
    inc.bent.assign((size_t)inc.bptr[n], 0);
    inc.tent.assign((size_t)inc.tptr[n], 0);
    std::vector<int> fill(inc.bptr.begin(), inc.bptr.end() - 1);
    if (use_bonds)
        for (int b = 0; b < n_edges; ++b) {
            inc.bent[fill[edge_ij[2 * b]]++] = (b << 1) | 0;
            inc.bent[fill[edge_ij[2 * b + 1]]++] = (b << 1) | 1;
        }
    fill.assign(inc.tptr.begin(), inc.tptr.end() - 1);
    if (use_triples)
        for (int t = 0; t < n_triples; ++t)
            for (int r = 0; r < 3; ++r) inc.tent[fill[tri_hjk[3 * t + r]]++] = (t << 2) | r;
}

}  // namespace nr

using nr::fail;

extern "C" {

const char *nr_status_string(int status) {
    switch (status) {
        case NR_OK: return "ok";
        case NR_NOT_CONVERGED: return "not converged (step cap reached)";
        case NR_ERR_INVALID: return "invalid argument";
        case NR_ERR_IO: return "i/o error";
        case NR_ERR_PARSE: return "parse error";
        case NR_ERR_CUDA: return "CUDA error";
        case NR_ERR_OOM: return "device out of memory";
        case NR_ERR_NONFINITE: return "non-finite force or position";
        case NR_ERR_TIMEOUT: return "grid barrier timed out";
        case NR_ERR_CAPACITY: return "request exceeds fixed capacity";
        default: return "unknown status";
    }
}

const char *nr_last_error(void) { return nr::g_last_error.c_str(); }
int nr_abi_version(void) { return NR_ABI_VERSION; }

/* get_triples, large_strain_relax.cu:116-184.  Per-node adjacency in edge
 * order (forward wrap for the first endpoint, negated for the second),
 * hinges ascending, pairs i < j in list order, accepted when dot < 0 and
 * |dot^2 - |a|^2 |b|^2| < 1e-10. */
int nr_get_triples(nr_host_network *net) {
    if (!net) return fail(NR_ERR_INVALID, "nr_get_triples: null network");
    const int n = net->n_points, ne = net->n_edges();
    std::vector<int> start((size_t)n + 1, 0);
    for (int e = 0; e < ne; ++e) {
        start[net->edge_ij[2 * e] + 1]++;
        start[net->edge_ij[2 * e + 1] + 1]++;
    }
    for (int i = 0; i < n; ++i) start[i + 1] += start[i];
    std::vector<int> fill(start.begin(), start.end() - 1), nb((size_t)2 * ne);
    std::vector<signed char> nw((size_t)2 * ne);
    for (int e = 0; e < ne; ++e) {
        const int a = net->edge_ij[2 * e], b = net->edge_ij[2 * e + 1];
        const signed char w = net->edge_wrap[e];
        nb[fill[a]] = b;
        nw[fill[a]++] = w;
        nb[fill[b]] = a;
        nw[fill[b]++] = (signed char)(-w);
    }
    net->tri_hjk.clear();
    net->tri_wrap.clear();
    net->tri_kb.clear();
    net->tri_phi0.clear();
    const double *p = net->points.data();
    const double offset = net->offset;
    /* hinges in contiguous ranges on several threads, results concatenated
     * in hinge order: the same list as one pass */
    const char *env = getenv("NR_IO_THREADS");
    int threads = env ? atoi(env) : 0;
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    threads = std::max(1, std::min(threads, std::max(1, n / 16384)));
    std::vector<std::vector<int>> hjk(threads);
    std::vector<std::vector<signed char>> tw(threads);
    auto work = [&](int t) {
        const int h0 = (int)((long)n * t / threads), h1 = (int)((long)n * (t + 1) / threads);
        for (int h = h0; h < h1; ++h) {
            const double x = p[2 * h], y = p[2 * h + 1];
            for (int i = start[h]; i < start[h + 1]; ++i) {
                const int j = nb[i];
                const double dx2 = p[2 * j] + offset * nw[i] - x;
                const double dy2 = p[2 * j + 1] - y;
                for (int k2 = i + 1; k2 < start[h + 1]; ++k2) {
                    const int k = nb[k2];
                    const double dx3 = p[2 * k] + offset * nw[k2] - x;
                    const double dy3 = p[2 * k + 1] - y;
                    const double dot = dx2 * dx3 + dy2 * dy3;
                    const double mag_sq = (dx2 * dx2 + dy2 * dy2) * (dx3 * dx3 + dy3 * dy3);
                    if (dot < 0 && std::fabs(dot * dot - mag_sq) < 1e-10) {
                        hjk[t].push_back(h);
                        hjk[t].push_back(j);
                        hjk[t].push_back(k);
                        tw[t].push_back(nw[i]);
                        tw[t].push_back(nw[k2]);
                    }
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto &th : pool) th.join();
    for (int t = 0; t < threads; ++t) {
        net->tri_hjk.insert(net->tri_hjk.end(), hjk[t].begin(), hjk[t].end());
        net->tri_wrap.insert(net->tri_wrap.end(), tw[t].begin(), tw[t].end());
    }
    return NR_OK;
}

int nr_host_network_from_arrays(int n_points, const double *points, int n_edges, const int *edge_ij,
                                const double *edge_l0, const signed char *edge_wrap, double offset,
                                nr_host_network **out) {
    if (!out || n_points <= 0 || n_edges < 0 || !points || (n_edges > 0 && (!edge_ij || !edge_wrap)))
        return fail(NR_ERR_INVALID, "nr_host_network_from_arrays: bad arguments");
    for (int e = 0; e < 2 * n_edges; ++e)
        if (edge_ij[e] < 0 || edge_ij[e] >= n_points)
            return fail(NR_ERR_INVALID, "nr_host_network_from_arrays: edge index out of range");
    auto *net = new nr_host_network();
    net->n_points = n_points;
    net->offset = offset;
    net->points.assign(points, points + 2 * (size_t)n_points);
    nr::y_range(net->points, net->miny, net->maxy);
    net->edge_ij.assign(edge_ij, edge_ij + 2 * (size_t)n_edges);
    net->edge_wrap.assign(edge_wrap, edge_wrap + n_edges);
    net->edge_l0.resize(n_edges);
    for (int e = 0; e < n_edges; ++e) {
        if (edge_l0) {
            net->edge_l0[e] = edge_l0[e];
        } else {
            const int i1 = edge_ij[2 * e], i2 = edge_ij[2 * e + 1];
            const double dx = points[2 * i2] + offset * edge_wrap[e] - points[2 * i1];
            const double dy = points[2 * i2 + 1] - points[2 * i1 + 1];
            net->edge_l0[e] = std::sqrt(dx * dx + dy * dy);
        }
    }
    *out = net;
    return NR_OK;
}

int nr_host_network_set_triples(nr_host_network *net, int n_triples, const int *tri_hjk, const signed char *tri_wrap,
                                const double *tri_kb, const double *tri_phi0) {
    if (!net || n_triples < 0 || (n_triples > 0 && (!tri_hjk || !tri_wrap)))
        return fail(NR_ERR_INVALID, "nr_host_network_set_triples: bad arguments");
    for (int i = 0; i < 3 * n_triples; ++i)
        if (tri_hjk[i] < 0 || tri_hjk[i] >= net->n_points)
            return fail(NR_ERR_INVALID, "nr_host_network_set_triples: node index out of range");
    net->tri_hjk.assign(tri_hjk, tri_hjk + 3 * (size_t)n_triples);
    net->tri_wrap.assign(tri_wrap, tri_wrap + 2 * (size_t)n_triples);
    if (tri_kb) net->tri_kb.assign(tri_kb, tri_kb + n_triples);
    else net->tri_kb.clear();
    if (tri_phi0) net->tri_phi0.assign(tri_phi0, tri_phi0 + n_triples);
    else net->tri_phi0.clear();
    return NR_OK;
}

int nr_host_network_set_bond_k(nr_host_network *net, const double *bond_k) {
    if (!net) return fail(NR_ERR_INVALID, "nr_host_network_set_bond_k: null network");
    if (bond_k) net->bond_k.assign(bond_k, bond_k + net->n_edges());
    else net->bond_k.clear();
    return NR_OK;
}

void nr_host_network_info(const nr_host_network *net, nr_host_info *info) {
    info->n_points = net->n_points;
    info->n_edges = net->n_edges();
    info->n_triples = net->n_triples();
    info->offset = net->offset;
    info->miny = net->miny;
    info->maxy = net->maxy;
    info->has_bond_k = !net->bond_k.empty();
    info->has_tri_kb = !net->tri_kb.empty();
    info->has_tri_phi0 = !net->tri_phi0.empty();
}

void nr_host_network_arrays(const nr_host_network *net, double *points, int *edge_ij, double *edge_l0,
                            signed char *edge_wrap, int *tri_hjk, signed char *tri_wrap, double *bond_k,
                            double *tri_kb, double *tri_phi0) {
    if (points) std::copy(net->points.begin(), net->points.end(), points);
    if (edge_ij) std::copy(net->edge_ij.begin(), net->edge_ij.end(), edge_ij);
    if (edge_l0) std::copy(net->edge_l0.begin(), net->edge_l0.end(), edge_l0);
    if (edge_wrap) std::copy(net->edge_wrap.begin(), net->edge_wrap.end(), edge_wrap);
    if (tri_hjk) std::copy(net->tri_hjk.begin(), net->tri_hjk.end(), tri_hjk);
    if (tri_wrap) std::copy(net->tri_wrap.begin(), net->tri_wrap.end(), tri_wrap);
    if (bond_k) std::copy(net->bond_k.begin(), net->bond_k.end(), bond_k);
    if (tri_kb) std::copy(net->tri_kb.begin(), net->tri_kb.end(), tri_kb);
    if (tri_phi0) std::copy(net->tri_phi0.begin(), net->tri_phi0.end(), tri_phi0);
}

void nr_host_network_fcodes(const nr_host_network *net, unsigned char *fcodes) {
    for (int i = 0; i < net->n_points; ++i) {
        const double y = net->points[2 * i + 1];
        fcodes[i] = (y < net->miny + 1e-10 || y > net->maxy - 1e-10) ? 0 : 3;
    }
}

void nr_host_network_free(nr_host_network *net) { delete net; }

}  // extern "C"
