/* Internal declarations shared by the host C++ and CUDA translation units. */
#ifndef NR_INTERNAL_H
#define NR_INTERNAL_H

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/netrelax.h"

struct nr_host_network {
    int n_points = 0;
    double offset = 0, miny = 0, maxy = 0;
    std::vector<double> points;       // 2N
    std::vector<int> edge_ij;         // 2E
    std::vector<double> edge_l0;      // E
    std::vector<signed char> edge_wrap;
    std::vector<int> tri_hjk;         // 3T
    std::vector<signed char> tri_wrap;// 2T
    std::vector<double> bond_k;       // empty or E
    std::vector<double> tri_kb;       // empty or T
    std::vector<double> tri_phi0;     // empty or T
    // network-mesh composites (network_mesh_relax.cu): FEM triangles, their
    // areas, pairs of duplicate vertices on the left / right edges, x range
    std::vector<int> facets;          // 3F
    std::vector<double> areas;        // F
    std::vector<int> mesh_pairs;      // 2P
    double minx = 0, maxx = 0;
    int n_edges() const { return (int)edge_l0.size(); }
    int n_triples() const { return (int)(tri_hjk.size() / 3); }
    int n_facets() const { return (int)(facets.size() / 3); }
    int n_mesh_pairs() const { return (int)(mesh_pairs.size() / 2); }
};

namespace nr {

/* Thread-local error message + status helper. */
int fail(int status, const std::string &msg);
void clear_error();

/* Per-node incidence lists in canonical order: every bond (in index order,
 * first endpoint before second) and every triple (in index order, hinge, j,
 * k) touching the node.  Entry encodings: bond (b << 1) | role,
 * triple (t << 2) | role. */
/* A launch-policy knob: the environment variable `name`, else the tuning
 * table's entry of that name (tuning.cu), else null. */
const char *knob(const char *name);

struct Incidence {
    std::vector<int> bptr, bent, tptr, tent;
};
void build_incidence(int n_points, const int *edge_ij, int n_edges, const int *tri_hjk, int n_triples, bool use_bonds,
                     bool use_triples, Incidence &inc);

/* Min/max y in the reader's convention (min starts at FLT_MAX, max at
 * FLT_MIN). */
void y_range(const std::vector<double> &points, double &miny, double &maxy);

/* n xy pairs written as "%2.10le\t%2.10le\n" lines (report_displaced,
 * large_strain_relax.cu:216-227), formatted in parallel. */
bool write_xy_file(const std::string &name, const double *xy, long n);

/* The duplicate-vertex search of read_network_mesh
 * (network_mesh_relax.cu:219-227): 2P indices. */
void find_mesh_pairs(const std::vector<double> &points, double offset, double minx, std::vector<int> &pairs);

}  // namespace nr

#endif
