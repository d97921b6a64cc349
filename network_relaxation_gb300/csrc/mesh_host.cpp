/*
 * Host side of network-mesh composites (network_mesh_relax.cu): the
 * duplicate-vertex search of read_network_mesh and the mesh accessors (the
 * .nmc reader and writer are in fast_io.cpp); and node reordering for
 * locality (Morton, RCM).
 */
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory_resource>
#include <string>
#include <vector>

#include "nr_internal.h"

namespace nr {

namespace {
constexpr double kPointTol = 1e-10; /* FLT_TOL, network_mesh_relax.cu:40 */

struct MeshPoint {
    double x, y;
};

/* PointComp (network_mesh_relax.cu:53-61): x with tolerance first, then y. */
struct MeshPointLess {
    bool operator()(const MeshPoint &a, const MeshPoint &b) const {
        if (a.x < b.x - kPointTol) return true;
        if (a.x > b.x + kPointTol) return false;
        return a.y < b.y - kPointTol;
    }
};
}  // namespace

/* The reader keeps the points in a std::map under PointComp (a point
 * equivalent to an earlier one is not inserted) and pairs every map entry
 * with x < minx + 1e-10, in map order, with the entry found at
 * (x + offset, y). */
void find_mesh_pairs(const std::vector<double> &points, double offset, double minx, std::vector<int> &pairs) {
    /* The same red-black tree as std::map (hence the same answers on
     * near-duplicates, where PointComp is not a strict order), with its
     * nodes carved from one buffer instead of one allocation each. */
    std::pmr::monotonic_buffer_resource arena(64 * (points.size() / 2 + 16));
    std::pmr::map<MeshPoint, int, MeshPointLess> pmap(&arena);
    for (size_t i = 0; i + 1 < points.size(); i += 2) pmap.insert({MeshPoint{points[i], points[i + 1]}, (int)(i / 2)});
    pairs.clear();
    for (auto it = pmap.begin(); it != pmap.end() && it->first.x < minx + kPointTol; ++it) {
        auto hit = pmap.find(MeshPoint{it->first.x + offset, it->first.y});
        if (hit != pmap.end()) {
            pairs.push_back(it->second);
            pairs.push_back(hit->second);
        }
    }
}

}  // namespace nr

using nr::fail;

extern "C" {

int nr_host_network_set_mesh(nr_host_network *net, int n_facets, const int *facets, const double *areas, int n_pairs,
                             const int *mesh_pairs) {
    if (!net || n_facets < 0 || (n_facets > 0 && (!facets || !areas)) || (n_pairs > 0 && !mesh_pairs))
        return fail(NR_ERR_INVALID, "nr_host_network_set_mesh: bad arguments");
    for (int i = 0; i < 3 * n_facets; ++i)
        if (facets[i] < 0 || facets[i] >= net->n_points)
            return fail(NR_ERR_INVALID, "nr_host_network_set_mesh: facet index out of range");
    for (int i = 0; i < n_facets; ++i)
        if (!(areas[i] > 0)) return fail(NR_ERR_INVALID, "nr_host_network_set_mesh: areas must be positive");
    for (int i = 0; i < 2 * n_pairs; ++i)
        if (mesh_pairs[i] < 0 || mesh_pairs[i] >= net->n_points)
            return fail(NR_ERR_INVALID, "nr_host_network_set_mesh: pair index out of range");
    net->facets.assign(facets, facets + 3 * (size_t)n_facets);
    net->areas.assign(areas, areas + n_facets);
    net->minx = FLT_MAX;
    net->maxx = FLT_MIN;
    for (int i = 0; i < net->n_points; ++i) {
        net->minx = std::min(net->minx, net->points[2 * i]);
        net->maxx = std::max(net->maxx, net->points[2 * i]);
    }
    if (n_pairs >= 0) net->mesh_pairs.assign(mesh_pairs, mesh_pairs + 2 * (size_t)n_pairs);
    else nr::find_mesh_pairs(net->points, net->offset, net->minx, net->mesh_pairs);
    return NR_OK;
}

int nr_host_network_set_offset(nr_host_network *net, double offset) {
    if (!net || !(offset >= 0)) return fail(NR_ERR_INVALID, "nr_host_network_set_offset: bad arguments");
    net->offset = offset;
    return NR_OK;
}

void nr_host_network_mesh_info(const nr_host_network *net, nr_mesh_info *info) {
    info->n_facets = net->n_facets();
    info->n_areas = (int)net->areas.size();
    info->n_mesh_pairs = net->n_mesh_pairs();
    info->minx = net->minx;
    info->maxx = net->maxx;
}

void nr_host_network_mesh_arrays(const nr_host_network *net, int *facets, double *areas, int *mesh_pairs) {
    if (facets) std::copy(net->facets.begin(), net->facets.end(), facets);
    if (areas) std::copy(net->areas.begin(), net->areas.end(), areas);
    if (mesh_pairs) std::copy(net->mesh_pairs.begin(), net->mesh_pairs.end(), mesh_pairs);
}

}  // extern "C"

/* ------------------------------------------------------ node reordering */

namespace {

/* Z-order key of a point on a 2^16 x 2^16 grid over the bounding box. */
uint32_t morton_key(double x, double y, double x0, double y0, double sx, double sy) {
    auto q = [](double v) -> uint32_t {
        if (!(v > 0)) return 0;
        if (v >= 65535.0) return 65535;
        return (uint32_t)v;
    };
    auto spread = [](uint32_t v) {
        v = (v | (v << 8)) & 0x00FF00FFu;
        v = (v | (v << 4)) & 0x0F0F0F0Fu;
        v = (v | (v << 2)) & 0x33333333u;
        v = (v | (v << 1)) & 0x55555555u;
        return v;
    };
    return spread(q((x - x0) * sx)) | (spread(q((y - y0) * sy)) << 1);
}

/* Reverse Cuthill-McKee on the bond graph: breadth-first from a
 * pseudo-peripheral node of every component (components in order of their
 * lowest node), neighbours by increasing degree, then reversed. */
std::vector<int> rcm_order(const nr_host_network &h) {
    const int n = h.n_points;
    std::vector<int> start(n + 1, 0);
    for (int e = 0; e < h.n_edges(); ++e) {
        start[h.edge_ij[2 * e] + 1]++;
        start[h.edge_ij[2 * e + 1] + 1]++;
    }
    for (int i = 0; i < n; ++i) start[i + 1] += start[i];
    std::vector<int> adj(start[n]), fill(start.begin(), start.end() - 1);
    for (int e = 0; e < h.n_edges(); ++e) {
        const int a = h.edge_ij[2 * e], b = h.edge_ij[2 * e + 1];
        adj[fill[a]++] = b;
        adj[fill[b]++] = a;
    }
    auto deg = [&](int v) { return start[v + 1] - start[v]; };
    for (int v = 0; v < n; ++v)
        std::stable_sort(adj.begin() + start[v], adj.begin() + start[v + 1],
                         [&](int a, int b) { return deg(a) < deg(b); });
    std::vector<int> order, level(n, -1);
    order.reserve(n);
    std::vector<char> seen(n, 0);
    auto bfs = [&](int root, std::vector<int> &out) { /* returns the last level's first node */
        out.clear();
        std::vector<int> q{root};
        level[root] = 0;
        size_t head = 0;
        while (head < q.size()) {
            const int v = q[head++];
            out.push_back(v);
            for (int k = start[v]; k < start[v + 1]; ++k)
                if (level[adj[k]] < 0) {
                    level[adj[k]] = level[v] + 1;
                    q.push_back(adj[k]);
                }
        }
        int far = root;
        for (int v : out)
            if (level[v] > level[far] || (level[v] == level[far] && deg(v) < deg(far))) far = v;
        for (int v : out) level[v] = -1;
        return far;
    };
    std::vector<int> comp;
    for (int s = 0; s < n; ++s) {
        if (seen[s]) continue;
        int root = s;
        for (int it = 0; it < 2; ++it) root = bfs(root, comp); /* two sweeps: a pseudo-peripheral node */
        bfs(root, comp);
        for (int v : comp) seen[v] = 1;
        order.insert(order.end(), comp.begin(), comp.end());
    }
    std::reverse(order.begin(), order.end());
    return order;
}

}  // namespace

extern "C" int nr_host_network_reorder(nr_host_network *net, int method, int *new_to_old) {
    if (!net || net->n_points <= 0 || (method != NR_ORDER_MORTON && method != NR_ORDER_RCM))
        return fail(NR_ERR_INVALID, "nr_host_network_reorder: bad arguments");
    const int n = net->n_points;
    std::vector<int> order(n); /* new position -> old node */
    if (method == NR_ORDER_MORTON) {
        double x0 = net->points[0], x1 = x0, y0 = net->points[1], y1 = y0;
        for (int i = 0; i < n; ++i) {
            x0 = std::min(x0, net->points[2 * i]);
            x1 = std::max(x1, net->points[2 * i]);
            y0 = std::min(y0, net->points[2 * i + 1]);
            y1 = std::max(y1, net->points[2 * i + 1]);
        }
        const double sx = x1 > x0 ? 65535.0 / (x1 - x0) : 0.0, sy = y1 > y0 ? 65535.0 / (y1 - y0) : 0.0;
        std::vector<uint32_t> key(n);
        for (int i = 0; i < n; ++i) {
            key[i] = morton_key(net->points[2 * i], net->points[2 * i + 1], x0, y0, sx, sy);
            order[i] = i;
        }
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] < key[b]; });
    } else {
        order = rcm_order(*net);
    }
    std::vector<int> old_to_new(n);
    for (int k = 0; k < n; ++k) old_to_new[order[k]] = k;
    std::vector<double> pts(2 * (size_t)n);
    for (int k = 0; k < n; ++k) {
        pts[2 * k] = net->points[2 * order[k]];
        pts[2 * k + 1] = net->points[2 * order[k] + 1];
    }
    net->points.swap(pts);
    for (int &v : net->edge_ij) v = old_to_new[v];
    for (int &v : net->tri_hjk) v = old_to_new[v];
    for (int &v : net->facets) v = old_to_new[v];
    for (int &v : net->mesh_pairs) v = old_to_new[v];
    if (new_to_old) std::copy(order.begin(), order.end(), new_to_old);
    return NR_OK;
}
