/*
 * Host side of network-mesh composites (network_mesh_relax.cu): the .nmc
 * reader (read_network_mesh), its duplicate-vertex search, a writer, and
 * accessors.  Compiled with -ffp-contract=off, like the .dat reader, so
 * rest lengths round exactly as the reference's host code.
 */
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <string>

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
    std::map<MeshPoint, int, MeshPointLess> pmap;
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

/* read_network_mesh, network_mesh_relax.cu:72-230: header "N E F offset",
 * points, edges "i j wrap", facets "i j k", areas; std::getline / eof()
 * as the reference uses them, so short files fail at the same point.  On
 * NR_ERR_PARSE the partially read network is still returned. */
int nr_read_network_mesh(const char *path, nr_host_network **out) {
    if (!path || !out) return fail(NR_ERR_INVALID, "nr_read_network_mesh: null argument");
    *out = nullptr;
    std::ifstream input(path);
    if (!input.is_open()) return fail(NR_ERR_IO, std::string("cannot open ") + path);
    auto *net = new nr_host_network();
    *out = net;
    std::string line;
    int num_points = 0, num_edges = 0, num_facets = 0;
    double offset = 0;
    net->minx = FLT_MAX;
    net->miny = FLT_MAX;
    net->maxx = FLT_MIN;
    net->maxy = FLT_MIN;
    std::getline(input, line);
    const int num_read = sscanf(line.c_str(), "%d %d %d %lf", &num_points, &num_edges, &num_facets, &offset);
    if (num_read < 4 || offset < 0 || num_points <= 0 || num_edges < 0 || num_facets < 0)
        return fail(NR_ERR_PARSE, "Reading failed. The provided file has an invalid header.");
    net->offset = offset;
    while (!input.eof() && net->points.size() < 2 * (size_t)num_points) {
        double x, y;
        std::getline(input, line);
        if (sscanf(line.c_str(), "%lf %lf", &x, &y) == 2) {
            net->points.push_back(x);
            net->points.push_back(y);
            if (x < net->minx) net->minx = x;
            if (y < net->miny) net->miny = y;
            if (x > net->maxx) net->maxx = x;
            if (y > net->maxy) net->maxy = y;
        }
    }
    net->n_points = (int)(net->points.size() / 2);
    if (input.eof()) return fail(NR_ERR_PARSE, "Reading failed. Too few points were read.");
    while (!input.eof() && net->edge_l0.size() < (size_t)num_edges) {
        int i1, i2;
        signed char mult;
        std::getline(input, line);
        if (sscanf(line.c_str(), "%d %d %hhd\n", &i1, &i2, &mult) == 3) {
            if (std::min(i1, i2) > -1 && std::max(i1, i2) < num_points) {
                const double dx = net->points[2 * i2] + offset * mult - net->points[2 * i1];
                const double dy = net->points[2 * i2 + 1] - net->points[2 * i1 + 1];
                net->edge_ij.push_back(i1);
                net->edge_ij.push_back(i2);
                net->edge_l0.push_back(std::sqrt(dx * dx + dy * dy));
                net->edge_wrap.push_back(mult);
            } else {
                return fail(NR_ERR_PARSE, "Reading failed due to an out-of-bounds point index.");
            }
        }
    }
    if (net->edge_l0.size() < (size_t)num_edges) return fail(NR_ERR_PARSE, "Too few edges were read.");
    if (input.eof() && num_facets > 0) return fail(NR_ERR_PARSE, "The file ended before facets could be read.");
    auto in_bounds = [&](int v) { return v >= 0 && v <= num_points - 1; };
    while (!input.eof() && net->facets.size() < 3 * (size_t)num_facets) {
        int i1, i2, i3;
        std::getline(input, line);
        if (sscanf(line.c_str(), "%d %d %d\n", &i1, &i2, &i3) == 3) {
            if (in_bounds(i1) && in_bounds(i2) && in_bounds(i3)) {
                net->facets.push_back(i1);
                net->facets.push_back(i2);
                net->facets.push_back(i3);
            } else {
                return fail(NR_ERR_PARSE, "Reading failed due to an out-of-bounds point index.");
            }
        }
    }
    if (net->facets.size() < 3 * (size_t)num_facets) return fail(NR_ERR_PARSE, "Too few facets were read.");
    if (input.eof() && num_facets > 0) return fail(NR_ERR_PARSE, "The file ended before facets could be read.");
    while (!input.eof() && net->areas.size() < (size_t)num_facets) {
        double area;
        std::getline(input, line);
        if (sscanf(line.c_str(), "%lf", &area) == 1) {
            if (area > 0) net->areas.push_back(area);
            else return fail(NR_ERR_PARSE, "An illegal area was specified.");
        }
    }
    if (net->areas.size() < (size_t)num_facets) return fail(NR_ERR_PARSE, "Too few areas were specified.");
    nr::find_mesh_pairs(net->points, offset, net->minx, net->mesh_pairs);
    return NR_OK;
}

/* Writes the format nr_read_network_mesh reads (%.17g, round-trips). */
int nr_write_network_mesh(const nr_host_network *net, const char *path) {
    if (!net || !path) return fail(NR_ERR_INVALID, "nr_write_network_mesh: null argument");
    FILE *f = fopen(path, "w");
    if (!f) return fail(NR_ERR_IO, std::string("cannot write ") + path);
    fprintf(f, "%d %d %d %.17g\n", net->n_points, net->n_edges(), net->n_facets(), net->offset);
    for (int i = 0; i < net->n_points; ++i) fprintf(f, "%.17g %.17g\n", net->points[2 * i], net->points[2 * i + 1]);
    for (int e = 0; e < net->n_edges(); ++e)
        fprintf(f, "%d %d %d\n", net->edge_ij[2 * e], net->edge_ij[2 * e + 1], (int)net->edge_wrap[e]);
    for (int t = 0; t < net->n_facets(); ++t)
        fprintf(f, "%d %d %d\n", net->facets[3 * t], net->facets[3 * t + 1], net->facets[3 * t + 2]);
    for (int t = 0; t < net->n_facets(); ++t) fprintf(f, "%.17g\n", net->areas[t]);
    fclose(f);
    return NR_OK;
}

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
