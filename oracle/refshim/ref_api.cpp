/*
 * extern "C" entry points onto the reference's own large_strain_relax.cu
 * functions, compiled for the host through cuda_runtime.h / cublas_v2.h in
 * this directory (see oracle/build_ref.sh).  Used by the test suite and the
 * golden-fixture generator in THIS container only, to pin the oracle to the
 * reference's behaviour.  The reference's functions have C++ linkage; they are
 * declared below with the exact signatures of large_strain_relax.cu so the
 * linker resolves them from the separately compiled reference object.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <tuple>
#include <vector>

using namespace std;

typedef tuple<int, int, double, char> edge_datum;          // large_strain_relax.cu:33
typedef tuple<int, int, int, char, char> triple_datum;     // large_strain_relax.cu:34
typedef tuple<double, double, double> strain_range;        // large_strain_relax.cu:38

bool read_network(string file_name, double &offset, vector<double> &points, vector<edge_datum> &edges,
                  double &min_y, double &max_y);                                    // :42
vector<triple_datum> get_triples(vector<double> points, vector<edge_datum> edges, double offset);  // :116
bool parse_batch_file(string file_name, string &base_name, string &tag, double *ks, double *kb,
                      double fp_list[5], int *nmin, double *mass, double *fcut, int *nmax,
                      strain_range &compr, strain_range &shearr);                   // :297
void affine_displace(int npoints, double *points, double miny, double yrange, double xdisp,
                     double ydisp);                                                 // :527 (kernel)
bool run_fire_md(int num_dof, int npairs, int ntriples, double width, double ks, double kb, double *d_pos,
                 double *d_vel, double *d_forces, int *d_pair_list, double *d_lengths, char *d_e_offsets,
                 int *d_triples, char *d_t_offsets, unsigned char *d_fcodes, double fire_params[5],
                 double mass, double fcut, int max_steps, int nmin, dim3 e_grid, dim3 block, dim3 t_grid,
                 double report_data[3], int &step_count);                           // :596
void do_relaxation_run(string net_file, string log_name, string edata_name, string disp_base, double ks,
                       double kb, double fire_params[5], int nmin, double mass, double fcut, int n_steps,
                       dim3 block, strain_range compr, strain_range shearr, bool strain_mode,
                       bool itemize);                                               // :792
int lsr_reference_main(int argc, char **argv);                                      // :1047 (renamed main)

namespace {
struct RefNetwork {
    double offset = 0, miny = 0, maxy = 0;
    vector<double> points;
    vector<edge_datum> edges;
    vector<triple_datum> triples;
    bool ok = false;
};
}  // namespace

extern "C" {

/* Reads a .dat with the reference's read_network and (when want_triples)
 * builds triples with its get_triples.  Returns an opaque handle. */
void *ref_load_network(const char *path, int want_triples) {
    auto *net = new RefNetwork();
    net->ok = read_network(path, net->offset, net->points, net->edges, net->miny, net->maxy);
    if (want_triples) net->triples = get_triples(net->points, net->edges, net->offset);
    return net;
}

void ref_free_network(void *h) { delete static_cast<RefNetwork *>(h); }

int ref_network_info(void *h, int *n_points, int *n_edges, int *n_triples, double *offset, double *miny,
                     double *maxy) {
    auto *net = static_cast<RefNetwork *>(h);
    *n_points = (int)(net->points.size() / 2);
    *n_edges = (int)net->edges.size();
    *n_triples = (int)net->triples.size();
    *offset = net->offset;
    *miny = net->miny;
    *maxy = net->maxy;
    return net->ok ? 1 : 0;
}

void ref_network_arrays(void *h, double *points, int *edge_ij, double *edge_l0, signed char *edge_wrap,
                        int *tri_hjk, signed char *tri_wrap) {
    auto *net = static_cast<RefNetwork *>(h);
    copy(net->points.begin(), net->points.end(), points);
    for (size_t e = 0; e < net->edges.size(); ++e) {
        edge_ij[2 * e] = get<0>(net->edges[e]);
        edge_ij[2 * e + 1] = get<1>(net->edges[e]);
        edge_l0[e] = get<2>(net->edges[e]);
        edge_wrap[e] = (signed char)get<3>(net->edges[e]);
    }
    for (size_t t = 0; t < net->triples.size(); ++t) {
        tri_hjk[3 * t] = get<0>(net->triples[t]);
        tri_hjk[3 * t + 1] = get<1>(net->triples[t]);
        tri_hjk[3 * t + 2] = get<2>(net->triples[t]);
        tri_wrap[2 * t] = (signed char)get<3>(net->triples[t]);
        tri_wrap[2 * t + 1] = (signed char)get<4>(net->triples[t]);
    }
}

/* The reference's affine_displace kernel body over the reference's own grid
 * (num_dof/128 + 1 blocks of 128 threads, launched with npoints = num_dof as
 * at large_strain_relax.cu:928/:970).  pos holds n_points xy pairs and is
 * updated in place. */
void ref_affine_displace(int n_points, double *pos, double miny, double yrange, double xdisp, double ydisp) {
    const int num_dof = 2 * n_points;
    double *d_pos = nullptr;
    cudaMalloc((void **)&d_pos, sizeof(double) * num_dof);
    cudaMemcpy(d_pos, pos, sizeof(double) * num_dof, cudaMemcpyHostToDevice);
    dim3 block(128, 1);
    dim3 grid(num_dof / 128 + 1, 1);
    nr_ref_launch(grid, block, affine_displace, num_dof, d_pos, miny, yrange, xdisp, ydisp);
    cudaMemcpy(pos, d_pos, sizeof(double) * num_dof, cudaMemcpyDeviceToHost);
    cudaFree(d_pos);
}

/* One call of the reference's run_fire_md on host copies of the arrays.
 * pos (2*n_points) is updated in place; vel and forces come back too. */
int ref_run_fire_md(int n_points, int n_edges, int n_triples, double width, double ks, double kb,
                    double *pos, double *vel, double *forces, const int *edge_ij, const double *edge_l0,
                    const signed char *edge_wrap, const int *tri_hjk, const signed char *tri_wrap,
                    const unsigned char *fcodes, const double fire_params[5], double mass, double fcut,
                    int max_steps, int nmin, double report[3], int *steps) {
    const int num_dof = 2 * n_points;
    double *d_pos, *d_vel, *d_forces, *d_lengths;
    int *d_pairs, *d_triples;
    char *d_e_off, *d_t_off;
    unsigned char *d_fcodes;
    cudaMalloc((void **)&d_pos, sizeof(double) * num_dof);
    cudaMalloc((void **)&d_vel, sizeof(double) * num_dof);
    cudaMalloc((void **)&d_forces, sizeof(double) * num_dof);
    cudaMalloc((void **)&d_fcodes, n_points);
    cudaMalloc((void **)&d_pairs, sizeof(int) * 2 * (size_t)n_edges);
    cudaMalloc((void **)&d_lengths, sizeof(double) * (size_t)n_edges);
    cudaMalloc((void **)&d_e_off, (size_t)n_edges);
    cudaMalloc((void **)&d_triples, sizeof(int) * 3 * (size_t)n_triples);
    cudaMalloc((void **)&d_t_off, 2 * (size_t)n_triples);
    memcpy(d_pos, pos, sizeof(double) * num_dof);
    memcpy(d_fcodes, fcodes, n_points);
    memcpy(d_pairs, edge_ij, sizeof(int) * 2 * (size_t)n_edges);
    memcpy(d_lengths, edge_l0, sizeof(double) * (size_t)n_edges);
    memcpy(d_e_off, edge_wrap, (size_t)n_edges);
    memcpy(d_triples, tri_hjk, sizeof(int) * 3 * (size_t)n_triples);
    memcpy(d_t_off, tri_wrap, 2 * (size_t)n_triples);
    dim3 block(128, 1);
    dim3 e_grid(n_edges / 128 + 1, 1);
    dim3 t_grid(n_triples / 128 + 1, 1);
    double fp[5];
    for (int i = 0; i < 5; ++i) fp[i] = fire_params[i];
    int step_count = 0;
    bool ok = run_fire_md(num_dof, n_edges, n_triples, width, ks, kb, d_pos, d_vel, d_forces, d_pairs, d_lengths,
                          d_e_off, d_triples, d_t_off, d_fcodes, fp, mass, fcut, max_steps, nmin, e_grid, block,
                          t_grid, report, step_count);
    *steps = step_count;
    memcpy(pos, d_pos, sizeof(double) * num_dof);
    if (vel) memcpy(vel, d_vel, sizeof(double) * num_dof);
    if (forces) memcpy(forces, d_forces, sizeof(double) * num_dof);
    cudaFree(d_pos); cudaFree(d_vel); cudaFree(d_forces); cudaFree(d_fcodes);
    cudaFree(d_pairs); cudaFree(d_lengths); cudaFree(d_e_off); cudaFree(d_triples); cudaFree(d_t_off);
    return ok ? 1 : 0;
}

/* The reference's whole per-network driver: reads net_file, runs the
 * compression then shear protocol, writes the log, edata and .pos files. */
void ref_do_relaxation_run(const char *net_file, const char *log_name, const char *edata_name,
                           const char *disp_base, double ks, double kb, const double fire_params[5], int nmin,
                           double mass, double fcut, int n_steps, const double compr[3],
                           const double shear[3]) {
    double fp[5];
    for (int i = 0; i < 5; ++i) fp[i] = fire_params[i];
    do_relaxation_run(net_file, log_name, edata_name, disp_base, ks, kb, fp, nmin, mass, fcut, n_steps,
                      dim3(128, 1), make_tuple(compr[0], compr[1], compr[2]),
                      make_tuple(shear[0], shear[1], shear[2]), true, false);
}

/* The reference's batch-file parser.  Returns 1 when it accepts the file. */
int ref_parse_batch_file(const char *path, char *base_out, int base_cap, char *tag_out, int tag_cap,
                         double *ks, double *kb, double fp[5], int *nmin, double *mass, double *fcut,
                         int *nmax, double compr[3], double shear[3]) {
    string base, tag;
    strain_range c{0, 0, 0}, s{0, 0, 0};
    bool ok = parse_batch_file(path, base, tag, ks, kb, fp, nmin, mass, fcut, nmax, c, s);
    snprintf(base_out, base_cap, "%s", base.c_str());
    snprintf(tag_out, tag_cap, "%s", tag.c_str());
    compr[0] = get<0>(c); compr[1] = get<1>(c); compr[2] = get<2>(c);
    shear[0] = get<0>(s); shear[1] = get<1>(s); shear[2] = get<2>(s);
    return ok ? 1 : 0;
}

/* The reference's lsrelax command line (main renamed at compile time). */
int ref_lsrelax_main(int argc, char **argv) { return lsr_reference_main(argc, argv); }

}  // extern "C"
