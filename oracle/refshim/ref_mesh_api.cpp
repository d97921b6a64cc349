/*
 * extern "C" entry points onto the reference's own network_mesh_relax.cu
 * functions (network + FEM gel composites), compiled for the host through
 * cuda_runtime.h / cublas_v2.h in this directory (see oracle/build_ref.sh).
 * Used by the test suite and the golden-fixture generator in THIS container
 * only, to pin the oracle to the reference's behaviour.  The reference's
 * functions are declared with the exact signatures of network_mesh_relax.cu
 * so the linker resolves them from the separately compiled reference object.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <tuple>
#include <vector>

using namespace std;

typedef tuple<int, int, double, char> edge_datum;       // network_mesh_relax.cu:32
typedef tuple<int, int, int, char, char> triple_datum;  // :33
typedef tuple<double, double, double> strain_range;     // :37

bool read_network_mesh(string file_name, double &offset, vector<double> &points, vector<edge_datum> &edges,
                       vector<int> &facets, vector<double> &areas, vector<int> &mesh_pairs, double &min_x,
                       double &min_y, double &max_x, double &max_y);                  // :72
vector<triple_datum> get_triples(vector<double> points, vector<edge_datum> edges, double offset);  // :232
bool parse_batch_file(string file_name, string &base_name, string &tag, double *ks, double *kb, double *bmod,
                      double *smod, double *dilation, double fp_list[5], int *nmin, double *mass, double *fcut,
                      int *nmax, strain_range &compr, strain_range &shearr);         // :413
void get_inv_mats(int n_facets, double *pos, int *facets, double *inv_mats);         // :503 (kernel)
void axial_forces(double ks, int npairs, double width, double *pos, unsigned char *fcodes, int *pair_list,
                  double *lengths, char *wrap_codes, double *forces);                // :534 (kernel)
void bending_forces(double kb, int ntriples, double width, double *pos, unsigned char *fcodes,
                    int *triple_list, char *wrap_codes, double *forces);             // :565 (kernel)
void gel_energy(double smod, double bmod, double dilation, int nelems, double *pos, int *elems,
                double *inv_mats, double *areas, double *energies);                  // :674 (kernel)
void gel_forces(double smod, double bmod, double dilation, int nelems, double *pos, int *elems,
                double *inv_mats, double *areas, unsigned char *fcodes, double *forces);  // :702 (kernel)
void duplicate_forces(unsigned char *fcodes, double *forces, int *m_pairs, int npairs);  // :754 (kernel)
void dilate(int npoints, double *points, double minx, double miny, double dilation);  // :796 (kernel)
bool run_fire_md(int num_dof, int npairs, int ntriples, int nelems, double width, double ks, double kb,
                 double smod, double bmod, double dilation, double *d_pos, double *d_vel, double *d_forces,
                 int *d_pair_list, double *d_lengths, char *d_e_offsets, int *d_triples, char *d_t_offsets,
                 int *d_elems, double *d_areas, double *d_inv_mats, int *d_mpairs, int n_mpairs,
                 unsigned char *d_fcodes, double fire_params[5], double mass, double fcut, int max_steps,
                 int nmin, dim3 e_grid, dim3 block, dim3 t_grid, dim3 m_grid, dim3 mp_grid,
                 double report_data[4], int &step_count);                            // :865
void do_relaxation_run(string net_file, string log_name, string edata_name, string disp_base, double ks,
                       double kb, double bmod, double smod, double dilation, double fire_params[5], int nmin,
                       double mass, double fcut, int n_steps, dim3 block, strain_range compr,
                       strain_range shearr, bool strain_mode, bool itemize);        // :1095
int nmr_reference_main(int argc, char **argv);                                      // renamed main

namespace {
struct RefMesh {
    double offset = 0, minx = 0, miny = 0, maxx = 0, maxy = 0;
    vector<double> points, areas;
    vector<edge_datum> edges;
    vector<triple_datum> triples;
    vector<int> facets, pairs;
    bool ok = false;
};

/* Device-style copies of a model's arrays (host memory under the shim). */
struct RefModel {
    double *pos, *forces;
    int *pairs, *triples, *elems, *mpairs;
    double *lengths, *areas, *inv;
    char *e_off, *t_off;
    unsigned char *fcodes;
};

template <class T>
T *dev_copy(const T *src, size_t n) {
    T *p = nullptr;
    cudaMalloc((void **)&p, sizeof(T) * (n ? n : 1));
    if (n) memcpy(p, src, sizeof(T) * n);
    return p;
}

RefModel make_model(int n_points, int n_edges, int n_triples, int n_elems, int n_mpairs, const double *pos,
                    const int *edge_ij, const double *edge_l0, const signed char *edge_wrap, const int *tri_hjk,
                    const signed char *tri_wrap, const int *elems, const double *areas, const double *inv,
                    const int *mpairs, const unsigned char *fcodes) {
    RefModel m;
    m.pos = dev_copy(pos, 2 * (size_t)n_points);
    m.forces = nullptr;
    cudaMalloc((void **)&m.forces, sizeof(double) * 2 * (size_t)n_points);
    m.pairs = dev_copy(edge_ij, 2 * (size_t)n_edges);
    m.lengths = dev_copy(edge_l0, (size_t)n_edges);
    m.e_off = dev_copy((const char *)edge_wrap, (size_t)n_edges);
    m.triples = dev_copy(tri_hjk, 3 * (size_t)n_triples);
    m.t_off = dev_copy((const char *)tri_wrap, 2 * (size_t)n_triples);
    m.elems = dev_copy(elems, 3 * (size_t)n_elems);
    m.areas = dev_copy(areas, (size_t)n_elems);
    m.inv = dev_copy(inv, 6 * (size_t)n_elems);
    m.mpairs = dev_copy(mpairs, 2 * (size_t)n_mpairs);
    m.fcodes = dev_copy(fcodes, (size_t)n_points);
    return m;
}

void free_model(RefModel &m) {
    cudaFree(m.pos); cudaFree(m.forces); cudaFree(m.pairs); cudaFree(m.lengths); cudaFree(m.e_off);
    cudaFree(m.triples); cudaFree(m.t_off); cudaFree(m.elems); cudaFree(m.areas); cudaFree(m.inv);
    cudaFree(m.mpairs); cudaFree(m.fcodes);
}

dim3 grid_for(long items) { return dim3((unsigned)(items / 128 + 1), 1); }
}  // namespace

extern "C" {

/* read_network_mesh (+ get_triples when want_triples, with period
 * triple_offset, or the file's offset when triple_offset < 0;
 * do_relaxation_run passes the dilated offset, :1141-1144). */
void *ref_load_mesh(const char *path, int want_triples, double triple_offset) {
    auto *m = new RefMesh();
    m->ok = read_network_mesh(path, m->offset, m->points, m->edges, m->facets, m->areas, m->pairs, m->minx,
                              m->miny, m->maxx, m->maxy);
    if (want_triples) m->triples = get_triples(m->points, m->edges, triple_offset < 0 ? m->offset : triple_offset);
    return m;
}

void ref_free_mesh(void *h) { delete static_cast<RefMesh *>(h); }

/* counts[6] = {points, edges, triples, facets, pairs, areas}; box[5] =
 * {offset, minx, miny, maxx, maxy}.  Returns the reader's result. */
int ref_mesh_info(void *h, int *counts, double *box) {
    auto *m = static_cast<RefMesh *>(h);
    counts[0] = (int)(m->points.size() / 2);
    counts[1] = (int)m->edges.size();
    counts[2] = (int)m->triples.size();
    counts[3] = (int)(m->facets.size() / 3);
    counts[4] = (int)(m->pairs.size() / 2);
    counts[5] = (int)m->areas.size();
    box[0] = m->offset; box[1] = m->minx; box[2] = m->miny; box[3] = m->maxx; box[4] = m->maxy;
    return m->ok ? 1 : 0;
}

void ref_mesh_arrays(void *h, double *points, int *edge_ij, double *edge_l0, signed char *edge_wrap, int *tri_hjk,
                     signed char *tri_wrap, int *facets, double *areas, int *pairs) {
    auto *m = static_cast<RefMesh *>(h);
    copy(m->points.begin(), m->points.end(), points);
    for (size_t e = 0; e < m->edges.size(); ++e) {
        edge_ij[2 * e] = get<0>(m->edges[e]);
        edge_ij[2 * e + 1] = get<1>(m->edges[e]);
        edge_l0[e] = get<2>(m->edges[e]);
        edge_wrap[e] = (signed char)get<3>(m->edges[e]);
    }
    for (size_t t = 0; t < m->triples.size(); ++t) {
        tri_hjk[3 * t] = get<0>(m->triples[t]);
        tri_hjk[3 * t + 1] = get<1>(m->triples[t]);
        tri_hjk[3 * t + 2] = get<2>(m->triples[t]);
        tri_wrap[2 * t] = (signed char)get<3>(m->triples[t]);
        tri_wrap[2 * t + 1] = (signed char)get<4>(m->triples[t]);
    }
    copy(m->facets.begin(), m->facets.end(), facets);
    copy(m->areas.begin(), m->areas.end(), areas);
    copy(m->pairs.begin(), m->pairs.end(), pairs);
}

/* The get_inv_mats kernel over its launch grid. */
void ref_get_inv_mats(int n_points, int n_elems, const double *pos, const int *elems, double *inv) {
    double *d_pos = dev_copy(pos, 2 * (size_t)n_points);
    int *d_el = dev_copy(elems, 3 * (size_t)n_elems);
    double *d_inv = nullptr;
    cudaMalloc((void **)&d_inv, sizeof(double) * 6 * (size_t)(n_elems ? n_elems : 1));
    nr_ref_launch(grid_for(n_elems), dim3(128, 1), get_inv_mats, n_elems, d_pos, d_el, d_inv);
    memcpy(inv, d_inv, sizeof(double) * 6 * (size_t)n_elems);
    cudaFree(d_pos); cudaFree(d_el); cudaFree(d_inv);
}

/* The dilate kernel as do_relaxation_run launches it (npoints = num_dof). */
void ref_dilate(int n_points, double *pos, double minx, double miny, double factor) {
    double *d_pos = dev_copy(pos, 2 * (size_t)n_points);
    nr_ref_launch(grid_for(2L * n_points), dim3(128, 1), dilate, 2 * n_points, d_pos, minx, miny, factor);
    memcpy(pos, d_pos, sizeof(double) * 2 * (size_t)n_points);
    cudaFree(d_pos);
}

/* One force evaluation in run_fire_md's order (:897-913): axial (ks > 0),
 * bending (kb > 0), then gel_forces and duplicate_forces (bmod > 0). */
void ref_mesh_forces(int n_points, int n_edges, int n_triples, int n_elems, int n_mpairs, double width, double ks,
                     double kb, double smod, double bmod, double dilation, const double *pos, const int *edge_ij,
                     const double *edge_l0, const signed char *edge_wrap, const int *tri_hjk,
                     const signed char *tri_wrap, const int *elems, const double *areas, const double *inv,
                     const int *mpairs, const unsigned char *fcodes, double *forces) {
    RefModel m = make_model(n_points, n_edges, n_triples, n_elems, n_mpairs, pos, edge_ij, edge_l0, edge_wrap,
                            tri_hjk, tri_wrap, elems, areas, inv, mpairs, fcodes);
    cudaMemset(m.forces, 0, sizeof(double) * 2 * (size_t)n_points);
    dim3 block(128, 1);
    if (ks > 0)
        nr_ref_launch(grid_for(n_edges), block, axial_forces, ks, n_edges, width, m.pos, m.fcodes, m.pairs,
                      m.lengths, m.e_off, m.forces);
    if (kb > 0)
        nr_ref_launch(grid_for(n_triples), block, bending_forces, kb, n_triples, width, m.pos, m.fcodes, m.triples,
                      m.t_off, m.forces);
    if (bmod > 0) {
        nr_ref_launch(grid_for(n_elems), block, gel_forces, smod, bmod, dilation, n_elems, m.pos, m.elems, m.inv,
                      m.areas, m.fcodes, m.forces);
        nr_ref_launch(grid_for(n_mpairs), block, duplicate_forces, m.fcodes, m.forces, m.mpairs, n_mpairs);
    }
    memcpy(forces, m.forces, sizeof(double) * 2 * (size_t)n_points);
    free_model(m);
}

/* Per-element gel energies (the gel_energy kernel). */
void ref_gel_energies(int n_points, int n_elems, double smod, double bmod, double dilation, const double *pos,
                      const int *elems, const double *areas, const double *inv, double *energies) {
    double *d_pos = dev_copy(pos, 2 * (size_t)n_points);
    int *d_el = dev_copy(elems, 3 * (size_t)n_elems);
    double *d_a = dev_copy(areas, (size_t)n_elems);
    double *d_inv = dev_copy(inv, 6 * (size_t)n_elems);
    double *d_e = nullptr;
    cudaMalloc((void **)&d_e, sizeof(double) * (size_t)(n_elems ? n_elems : 1));
    nr_ref_launch(grid_for(n_elems), dim3(128, 1), gel_energy, smod, bmod, dilation, n_elems, d_pos, d_el, d_inv,
                  d_a, d_e);
    memcpy(energies, d_e, sizeof(double) * (size_t)n_elems);
    cudaFree(d_pos); cudaFree(d_el); cudaFree(d_a); cudaFree(d_inv); cudaFree(d_e);
}

/* One call of network_mesh_relax.cu's run_fire_md on host copies of the
 * arrays.  pos is updated in place; report[4] = {rms, E_s, E_b, E_gel}. */
int ref_mesh_run_fire_md(int n_points, int n_edges, int n_triples, int n_elems, int n_mpairs, double width,
                         double ks, double kb, double smod, double bmod, double dilation, double *pos,
                         const int *edge_ij, const double *edge_l0, const signed char *edge_wrap,
                         const int *tri_hjk, const signed char *tri_wrap, const int *elems, const double *areas,
                         const double *inv, const int *mpairs, const unsigned char *fcodes,
                         const double fire_params[5], double mass, double fcut, int max_steps, int nmin,
                         double report[4], int *steps) {
    RefModel m = make_model(n_points, n_edges, n_triples, n_elems, n_mpairs, pos, edge_ij, edge_l0, edge_wrap,
                            tri_hjk, tri_wrap, elems, areas, inv, mpairs, fcodes);
    double *d_vel = nullptr;
    cudaMalloc((void **)&d_vel, sizeof(double) * 2 * (size_t)n_points);
    double fp[5];
    for (int i = 0; i < 5; ++i) fp[i] = fire_params[i];
    int step_count = 0;
    dim3 block(128, 1);
    bool ok = run_fire_md(2 * n_points, n_edges, n_triples, n_elems, width, ks, kb, smod, bmod, dilation, m.pos,
                          d_vel, m.forces, m.pairs, m.lengths, m.e_off, m.triples, m.t_off, m.elems, m.areas, m.inv,
                          m.mpairs, n_mpairs, m.fcodes, fp, mass, fcut, max_steps, nmin, grid_for(n_edges), block,
                          grid_for(n_triples), grid_for(n_elems), grid_for(n_mpairs), report, step_count);
    *steps = step_count;
    memcpy(pos, m.pos, sizeof(double) * 2 * (size_t)n_points);
    cudaFree(d_vel);
    free_model(m);
    return ok ? 1 : 0;
}

/* The reference's whole per-network driver (network_mesh_relax.cu:1095),
 * strain mode: reads net_file, writes the log, edata and .pos files. */
void ref_mesh_do_relaxation_run(const char *net_file, const char *log_name, const char *edata_name,
                                const char *disp_base, double ks, double kb, double bmod, double smod,
                                double dilation, const double fire_params[5], int nmin, double mass, double fcut,
                                int n_steps, const double compr[3], const double shear[3]) {
    double fp[5];
    for (int i = 0; i < 5; ++i) fp[i] = fire_params[i];
    do_relaxation_run(net_file, log_name, edata_name, disp_base, ks, kb, bmod, smod, dilation, fp, nmin, mass, fcut,
                      n_steps, dim3(128, 1), make_tuple(compr[0], compr[1], compr[2]),
                      make_tuple(shear[0], shear[1], shear[2]), true, false);
}

/* The reference's batch-file parser; mech[5] = {ks, kb, bmod, smod,
 * dilation}.  Returns 1 when it accepts the file. */
int ref_mesh_parse_batch_file(const char *path, char *base_out, int base_cap, char *tag_out, int tag_cap,
                              double mech[5], double fp[5], int *nmin, double *mass, double *fcut, int *nmax,
                              double compr[3], double shear[3]) {
    string base, tag;
    strain_range c{0, 0, 0}, s{0, 0, 0};
    bool ok = parse_batch_file(path, base, tag, mech, mech + 1, mech + 2, mech + 3, mech + 4, fp, nmin, mass, fcut,
                               nmax, c, s);
    snprintf(base_out, base_cap, "%s", base.c_str());
    snprintf(tag_out, tag_cap, "%s", tag.c_str());
    compr[0] = get<0>(c); compr[1] = get<1>(c); compr[2] = get<2>(c);
    shear[0] = get<0>(s); shear[1] = get<1>(s); shear[2] = get<2>(s);
    return ok ? 1 : 0;
}

/* The reference's nmrelax command line (main renamed at compile time). */
int ref_nmrelax_main(int argc, char **argv) { return nmr_reference_main(argc, argv); }

}  // extern "C"
