/*
 * Dense stand-ins for the CHOLMOD / SPQR calls of the reference's
 * sparse_relax.cpp (declared in spr_include/SuiteSparseQR.hpp), and
 * extern "C" entry points onto that file's own functions, compiled for the
 * host by oracle/build_ref.sh.  Used by the test suite and the
 * golden-fixture generator in THIS container only, to pin the oracle to the
 * reference.  The reference's functions are declared with the exact
 * signatures of sparse_relax.cpp so the linker resolves them from its
 * separately compiled object.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <tuple>
#include <vector>

#include "SuiteSparseQR.hpp"
#include "cholmod_gpu.h"

using namespace std;

/* ------------------------------------------------------------ stand-ins */

int cholmod_l_start(cholmod_common *cc) {
    cc->useGPU = 0;
    cc->gpuMemorySize = 0;
    return 1;
}
int cholmod_l_finish(cholmod_common *) { return 1; }
int cholmod_l_gpu_memorysize(size_t *total, size_t *avail, cholmod_common *) {
    *total = *avail = 0;
    return 0;
}

cholmod_triplet *cholmod_l_allocate_triplet(size_t nrow, size_t ncol, size_t nzmax, int stype, int xtype,
                                            cholmod_common *) {
    auto *T = new cholmod_triplet();
    T->nrow = nrow;
    T->ncol = ncol;
    T->nzmax = nzmax;
    T->nnz = 0;
    T->stype = stype;
    T->itype = CHOLMOD_LONG;
    T->xtype = xtype;
    T->i = calloc(nzmax + 1, sizeof(SuiteSparse_long));
    T->j = calloc(nzmax + 1, sizeof(SuiteSparse_long));
    T->x = calloc(nzmax + 1, sizeof(double));
    return T;
}
int cholmod_l_free_triplet(cholmod_triplet **T, cholmod_common *) {
    if (*T) {
        free((*T)->i);
        free((*T)->j);
        free((*T)->x);
        delete *T;
        *T = nullptr;
    }
    return 1;
}

static cholmod_sparse *new_sparse(size_t nrow, size_t ncol) {
    auto *A = new cholmod_sparse();
    A->nrow = nrow;
    A->ncol = ncol;
    A->stype = 0;
    A->a = (double *)calloc(nrow * ncol + 1, sizeof(double));
    return A;
}
static double &at(cholmod_sparse *A, size_t i, size_t j) { return A->a[j * A->nrow + i]; }

/* Symmetric triplets (stype != 0) fill both triangles. */
cholmod_sparse *cholmod_l_triplet_to_sparse(cholmod_triplet *T, size_t, cholmod_common *) {
    cholmod_sparse *A = new_sparse(T->nrow, T->ncol);
    const SuiteSparse_long *ti = (const SuiteSparse_long *)T->i, *tj = (const SuiteSparse_long *)T->j;
    const double *tx = (const double *)T->x;
    for (size_t k = 0; k < T->nnz; ++k) {
        at(A, ti[k], tj[k]) += tx[k];
        if (T->stype != 0 && ti[k] != tj[k]) at(A, tj[k], ti[k]) += tx[k];
    }
    return A;
}
cholmod_sparse *cholmod_l_transpose(cholmod_sparse *A, int, cholmod_common *) {
    cholmod_sparse *B = new_sparse(A->ncol, A->nrow);
    for (size_t j = 0; j < A->ncol; ++j)
        for (size_t i = 0; i < A->nrow; ++i) at(B, j, i) = at(A, i, j);
    return B;
}
/* C = A B, each entry summed over k in increasing order. */
cholmod_sparse *cholmod_l_ssmult(cholmod_sparse *A, cholmod_sparse *B, int, int, int, cholmod_common *) {
    cholmod_sparse *C = new_sparse(A->nrow, B->ncol);
    for (size_t j = 0; j < B->ncol; ++j)
        for (size_t k = 0; k < A->ncol; ++k) {
            const double b = at(B, k, j);
            if (b == 0) continue;
            for (size_t i = 0; i < A->nrow; ++i) {
                const double a = at(A, i, k);
                if (a != 0) at(C, i, j) += a * b;
            }
        }
    return C;
}
int cholmod_l_free_sparse(cholmod_sparse **A, cholmod_common *) {
    if (*A) {
        free((*A)->a);
        delete *A;
        *A = nullptr;
    }
    return 1;
}
cholmod_dense *cholmod_l_zeros(size_t nrow, size_t ncol, int xtype, cholmod_common *) {
    auto *X = new cholmod_dense();
    X->nrow = nrow;
    X->ncol = ncol;
    X->nzmax = nrow * ncol;
    X->d = nrow;
    X->xtype = xtype;
    X->x = calloc(nrow * ncol + 1, sizeof(double));
    return X;
}
int cholmod_l_free_dense(cholmod_dense **X, cholmod_common *) {
    if (*X) {
        free((*X)->x);
        delete *X;
        *X = nullptr;
    }
    return 1;
}
/* Y = alpha op(A) X + beta Y (column vectors), column by column. */
int cholmod_l_sdmult(cholmod_sparse *A, int transpose, double alpha[2], double beta[2], cholmod_dense *X,
                     cholmod_dense *Y, cholmod_common *) {
    const size_t m = transpose ? A->ncol : A->nrow, n = transpose ? A->nrow : A->ncol;
    double *y = (double *)Y->x;
    const double *x = (const double *)X->x;
    for (size_t i = 0; i < m; ++i) y[i] = beta[0] == 0 ? 0.0 : beta[0] * y[i];
    for (size_t j = 0; j < n; ++j) {
        const double xj = alpha[0] * x[j];
        for (size_t i = 0; i < m; ++i) {
            const double a = transpose ? at(A, j, i) : at(A, i, j);
            if (a != 0) y[i] += a * xj;
        }
    }
    return 1;
}
int cholmod_l_copy_dense2(cholmod_dense *X, cholmod_dense *Y, cholmod_common *) {
    memcpy(Y->x, X->x, sizeof(double) * X->nrow * X->ncol);
    return 1;
}
double cholmod_l_norm_dense(cholmod_dense *X, int, cholmod_common *) {
    double s = 0;
    const double *x = (const double *)X->x;
    for (size_t i = 0; i < X->nrow; ++i) s += x[i] * x[i];
    return sqrt(s);
}
int cholmod_l_print_sparse(cholmod_sparse *, const char *, cholmod_common *) { return 1; }

[[noreturn]] static void unsupported(const char *what) {
    fprintf(stderr, "refshim: %s is not provided (only reached with -n)\n", what);
    abort();
}
cholmod_sparse *cholmod_l_spzeros(size_t, size_t, size_t, int, cholmod_common *) { unsupported("spzeros"); }
cholmod_sparse *cholmod_l_speye(size_t, size_t, int, cholmod_common *) { unsupported("speye"); }
cholmod_sparse *cholmod_l_vertcat(cholmod_sparse *, cholmod_sparse *, int, cholmod_common *) { unsupported("vertcat"); }
cholmod_sparse *cholmod_l_horzcat(cholmod_sparse *, cholmod_sparse *, int, cholmod_common *) { unsupported("horzcat"); }
cholmod_sparse *cholmod_l_submatrix(cholmod_sparse *, SuiteSparse_long *, SuiteSparse_long, SuiteSparse_long *,
                                    SuiteSparse_long, int, int, cholmod_common *) {
    unsupported("submatrix");
}
template <>
SuiteSparseQR_factorization<double> *SuiteSparseQR_factorize<double>(int, double, cholmod_sparse *, cholmod_common *) {
    unsupported("SuiteSparseQR_factorize");
}
template <>
cholmod_sparse *SuiteSparseQR_qmult<double>(int, SuiteSparseQR_factorization<double> *, cholmod_sparse *,
                                            cholmod_common *) {
    unsupported("SuiteSparseQR_qmult");
}
template <>
void SuiteSparseQR_free<double>(SuiteSparseQR_factorization<double> **, cholmod_common *) {
    unsupported("SuiteSparseQR_free");
}

/* x = A \ b for square A by Gaussian elimination with partial pivoting; a
 * column without a usable pivot (rank deficiency) gets x = 0 there. */
template <>
cholmod_dense *SuiteSparseQR<double>(cholmod_sparse *A, cholmod_dense *B, cholmod_common *cc) {
    const size_t n = A->nrow;
    vector<double> M(A->a, A->a + n * A->ncol), b((double *)B->x, (double *)B->x + n);
    vector<size_t> piv_col;
    vector<char> used(n, 0);
    vector<long> pivot_row_of_col(n, -1);
    double scale = 0;
    for (double v : M) scale = fmax(scale, fabs(v));
    size_t r = 0;
    for (size_t c = 0; c < A->ncol && r < n; ++c) {
        size_t best = r;
        for (size_t i = r + 1; i < n; ++i)
            if (fabs(M[c * n + i]) > fabs(M[c * n + best])) best = i;
        if (!(fabs(M[c * n + best]) > 1e-13 * scale)) continue;
        if (best != r) {
            for (size_t k = 0; k < A->ncol; ++k) std::swap(M[k * n + r], M[k * n + best]);
            std::swap(b[r], b[best]);
        }
        for (size_t i = r + 1; i < n; ++i) {
            const double f = M[c * n + i] / M[c * n + r];
            if (f == 0) continue;
            for (size_t k = c; k < A->ncol; ++k) M[k * n + i] -= f * M[k * n + r];
            b[i] -= f * b[r];
        }
        pivot_row_of_col[c] = (long)r;
        ++r;
    }
    cholmod_dense *X = cholmod_l_zeros(A->ncol, 1, CHOLMOD_REAL, cc);
    double *x = (double *)X->x;
    for (long c = (long)A->ncol - 1; c >= 0; --c) {
        const long pr = pivot_row_of_col[c];
        if (pr < 0) continue;
        double s = b[pr];
        for (size_t k = c + 1; k < A->ncol; ++k) s -= M[k * n + pr] * x[k];
        x[c] = s / M[c * n + pr];
    }
    return X;
}

/* ------------------------------------------- the reference's own functions */

typedef tuple<double, double> vec2d;                   // sparse_relax.cpp:41
typedef tuple<int, int, double, char> edge_datum;      // :42
typedef tuple<int, int, int, char> triple_datum;       // :43

bool read_network(ifstream &input, double &offset, vector<vec2d> &points, vector<edge_datum> &edges,
                  double &min_x, double &max_x, double &min_y, double &max_y);          // :114
vector<triple_datum> get_triples(vector<vec2d> points, vector<edge_datum> edges, double offset);  // :196
cholmod_sparse *get_sparse_stiffness_mat(vector<vec2d> points, vector<edge_datum> edges, vector<triple_datum> &tdata,
                                         double offset, double ks, double kb, double mu, cholmod_common *cc);  // :434
void get_stretch_shear_energy(vector<vec2d> points, vector<edge_datum> edges, double offset, cholmod_dense *u,
                              double ks, double mu, double &e_ss);                     // :49
void get_bending_energy(vector<vec2d> points, vector<triple_datum> tdata, double offset, cholmod_dense *u,
                        double kb, double &e_bend);                                     // :74
bool parse_batch_file(string file_name, string &base_name, string &tag, double &ks, double &kb, double &mu,
                      double &cmin, double &cmax, double &cinc, double &smin, double &smax, double &sinc);  // :931
void do_relaxation_run(string dat_name, string log_name, string disp_base, string e_name, double ks, double kb,
                       double mu, double min_c, double max_c, double c_inc, double min_s, double max_s,
                       double s_inc, bool strain_mode, bool affine, bool remove_np, bool itemize,
                       cholmod_common *cc);                                              // :676
int spr_reference_main(int argc, char **argv);                                           // renamed main

namespace {
struct RefSpr {
    double offset = 0, minx = 0, maxx = 0, miny = 0, maxy = 0;
    vector<vec2d> points;
    vector<edge_datum> edges;
    vector<triple_datum> triples;
    bool ok = false;
};
}  // namespace

extern "C" {

/* read_network (SPR's own) + get_triples (SPR's own, one wrap per triple). */
void *ref_spr_load(const char *path) {
    auto *m = new RefSpr();
    ifstream input(path);
    if (input.is_open()) {
        m->ok = read_network(input, m->offset, m->points, m->edges, m->minx, m->maxx, m->miny, m->maxy);
        m->triples = get_triples(m->points, m->edges, m->offset);
    }
    return m;
}
void ref_spr_free(void *h) { delete static_cast<RefSpr *>(h); }
/* counts[3] = {points, edges, triples}; box[5] = {offset, minx, maxx, miny, maxy} */
int ref_spr_info(void *h, int *counts, double *box) {
    auto *m = static_cast<RefSpr *>(h);
    counts[0] = (int)m->points.size();
    counts[1] = (int)m->edges.size();
    counts[2] = (int)m->triples.size();
    box[0] = m->offset; box[1] = m->minx; box[2] = m->maxx; box[3] = m->miny; box[4] = m->maxy;
    return m->ok ? 1 : 0;
}
void ref_spr_arrays(void *h, double *points, int *edge_ij, double *edge_l0, signed char *edge_wrap, int *tri_hjk,
                    signed char *tri_wrap) {
    auto *m = static_cast<RefSpr *>(h);
    for (size_t i = 0; i < m->points.size(); ++i) {
        points[2 * i] = get<0>(m->points[i]);
        points[2 * i + 1] = get<1>(m->points[i]);
    }
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
        tri_wrap[t] = (signed char)get<3>(m->triples[t]);
    }
}
/* get_sparse_stiffness_mat on the loaded network: the nonzero entries of
 * its upper triangle in (row, col) order; returns their number (arrays may
 * be NULL to count). */
long ref_spr_stiffness(void *h, double ks, double kb, double mu, long *rows, long *cols, double *vals) {
    auto *m = static_cast<RefSpr *>(h);
    cholmod_common cc;
    cholmod_l_start(&cc);
    vector<triple_datum> tdata;
    cholmod_sparse *K = get_sparse_stiffness_mat(m->points, m->edges, tdata, m->offset, ks, kb, mu, &cc);
    long nnz = 0;
    for (size_t i = 0; i < K->nrow; ++i)
        for (size_t j = i; j < K->ncol; ++j) {
            const double v = K->a[j * K->nrow + i];
            if (v != 0) {
                if (rows) {
                    rows[nnz] = (long)i;
                    cols[nnz] = (long)j;
                    vals[nnz] = v;
                }
                nnz++;
            }
        }
    cholmod_l_free_sparse(&K, &cc);
    return nnz;
}
/* The linearised energies of a full displacement field u (2N). */
void ref_spr_energies(void *h, double ks, double kb, double mu, const double *u, double *e_ss, double *e_bend) {
    auto *m = static_cast<RefSpr *>(h);
    cholmod_common cc;
    cholmod_dense *U = cholmod_l_zeros(2 * m->points.size(), 1, CHOLMOD_REAL, &cc);
    memcpy(U->x, u, sizeof(double) * 2 * m->points.size());
    *e_ss = 0;
    *e_bend = 0;
    if (ks > 0 || mu > 0) get_stretch_shear_energy(m->points, m->edges, m->offset, U, ks, mu, *e_ss);
    if (kb > 0) get_bending_energy(m->points, m->triples, m->offset, U, kb, *e_bend);
    cholmod_l_free_dense(&U, &cc);
}
/* The reference's per-network driver (SPR:676); names may be empty. */
void ref_spr_do_relaxation_run(const char *dat, const char *log, const char *disp_base, const char *e_name, double ks,
                               double kb, double mu, const double c[3], const double s[3], int strain_mode, int affine,
                               int itemize) {
    cholmod_common cc;
    cholmod_l_start(&cc);
    do_relaxation_run(dat, log, disp_base, e_name, ks, kb, mu, c[0], c[1], c[2], s[0], s[1], s[2], strain_mode != 0,
                      affine != 0, false, itemize != 0, &cc);
}
int ref_spr_parse_batch_file(const char *path, char *base_out, int base_cap, char *tag_out, int tag_cap,
                             double mech[3], double c[3], double s[3]) {
    string base, tag;
    bool ok = parse_batch_file(path, base, tag, mech[0], mech[1], mech[2], c[0], c[1], c[2], s[0], s[1], s[2]);
    snprintf(base_out, base_cap, "%s", base.c_str());
    snprintf(tag_out, tag_cap, "%s", tag.c_str());
    return ok ? 1 : 0;
}
int ref_spr_main(int argc, char **argv) { return spr_reference_main(argc, argv); }

}  // extern "C"
