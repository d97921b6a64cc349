/*
 * nr_oracle_spr.c — CPU restatement of the linear-response solve of
 * src/sparse_relax.cpp (SPR): the stiffness matrix of stretching, linearised
 * bending and background shear, the projection onto the free nodes, the
 * boundary-condition vectors and the linearised energies.
 * TEST INFRASTRUCTURE ONLY (see nr_oracle.h).  Compile with
 * -ffp-contract=off; every expression keeps the reference's association.
 *
 * The sparse solve itself is SuiteSparseQR's (SuiteSparse SPQR, absent
 * here); the Python side of the oracle restates it as a dense least-squares
 * solve (for a full-rank system both are the unique solution).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "nr_oracle.h"

#define OR_SPR_TOL 1e-10 /* FLT_TOL, sparse_relax.cpp:45 */

typedef struct {
    long i, j, seq;
    double v;
} or_contrib;

typedef struct {
    or_contrib *c;
    long n, cap;
} or_contribs;

/* update_matrix (SPR:268-277): the key is the ordered index pair. */
static void or_update(or_contribs *s, long a, long b, double v) {
    if (s->n == s->cap) {
        s->cap = s->cap ? 2 * s->cap : 1024;
        s->c = (or_contrib *)realloc(s->c, sizeof(or_contrib) * (size_t)s->cap);
    }
    or_contrib *e = s->c + s->n;
    e->i = a < b ? a : b;
    e->j = a < b ? b : a;
    e->seq = s->n;
    e->v = v;
    s->n++;
}

static int or_contrib_cmp(const void *pa, const void *pb) {
    const or_contrib *a = (const or_contrib *)pa, *b = (const or_contrib *)pb;
    if (a->i != b->i) return a->i < b->i ? -1 : 1;
    if (a->j != b->j) return a->j < b->j ? -1 : 1;
    return a->seq < b->seq ? -1 : (a->seq > b->seq);
}

/* get_sparse_stiffness_mat (SPR:434-480) with calc_stretching_elements
 * (:280-323), calc_bending_elements (:326-386, kb > 0) and
 * calc_shearing_elements (:390-429, mu > 0).  The reference accumulates in
 * a std::map keyed by (row <= col): a key's value is its contributions
 * added in call order.  Entries with |value| <= 1e-10 are dropped.  Output:
 * the upper-triangle triplets in (row, col) order; returns their number.
 * tri_wrap holds 2 per triple; SPR's triples keep only the first (hinge to
 * j, :257). */
long or_spr_stiffness(int n_points, const double *p, int n_edges, const int *edge_ij, const double *edge_l0,
                      const signed char *edge_wrap, double offset, double ks, double kb, double mu, int n_triples,
                      const int *tri_hjk, const signed char *tri_wrap, long *rows, long *cols, double *vals) {
    (void)n_points;
    or_contribs s = {NULL, 0, 0};
    for (int e = 0; e < n_edges; ++e) {
        const int a = edge_ij[2 * e], b = edge_ij[2 * e + 1];
        const double dx = p[2 * b] + offset * edge_wrap[e] - p[2 * a];
        const double dy = p[2 * b + 1] - p[2 * a + 1];
        const double l = sqrt(dx * dx + dy * dy);
        const double inv_l_cubed = 1 / (l * l * l);
        const long x1 = 2L * a, x2 = 2L * b, y1 = 2L * a + 1, y2 = 2L * b + 1;
        double m = ks * inv_l_cubed * dx * dx;
        or_update(&s, x1, x2, -m);
        or_update(&s, x1, x1, m);
        or_update(&s, x2, x2, m);
        m = ks * inv_l_cubed * dx * dy;
        or_update(&s, x1, y2, -m);
        or_update(&s, y1, x2, -m);
        or_update(&s, x1, y1, m);
        or_update(&s, x2, y2, m);
        m = ks * inv_l_cubed * dy * dy;
        or_update(&s, y1, y2, -m);
        or_update(&s, y1, y1, m);
        or_update(&s, y2, y2, m);
    }
    if (kb > 0) {
        for (int t = 0; t < n_triples; ++t) {
            const long h = tri_hjk[3 * t], j = tri_hjk[3 * t + 1], k = tri_hjk[3 * t + 2];
            const double dx = p[2 * j] + offset * tri_wrap[2 * t] - p[2 * h];
            const double dy = p[2 * j + 1] - p[2 * h + 1];
            const double len_sq = dx * dx + dy * dy;
            const double xx = kb * dx * dx / len_sq;
            const double yy = kb * dy * dy / len_sq;
            const double xy = kb * dx * dy / len_sq;
            or_update(&s, 2 * h, 2 * h, 4 * yy);
            or_update(&s, 2 * j, 2 * j, yy);
            or_update(&s, 2 * k, 2 * k, yy);
            or_update(&s, 2 * h + 1, 2 * h + 1, 4 * xx);
            or_update(&s, 2 * j + 1, 2 * j + 1, xx);
            or_update(&s, 2 * k + 1, 2 * k + 1, xx);
            or_update(&s, 2 * h, 2 * h + 1, -4 * xy);
            or_update(&s, 2 * h, 2 * j, -2 * yy);
            or_update(&s, 2 * h, 2 * k, -2 * yy);
            or_update(&s, 2 * h, 2 * j + 1, 2 * xy);
            or_update(&s, 2 * h, 2 * k + 1, 2 * xy);
            or_update(&s, 2 * h + 1, 2 * j, 2 * xy);
            or_update(&s, 2 * h + 1, 2 * k, 2 * xy);
            or_update(&s, 2 * h + 1, 2 * j + 1, -2 * xx);
            or_update(&s, 2 * h + 1, 2 * k + 1, -2 * xx);
            or_update(&s, j * 2, j * 2 + 1, -xy);
            or_update(&s, j * 2, k * 2, yy);
            or_update(&s, j * 2, k * 2 + 1, -xy);
            or_update(&s, j * 2 + 1, k * 2, -xy);
            or_update(&s, j * 2 + 1, k * 2 + 1, xx);
            or_update(&s, k * 2, k * 2 + 1, -xy);
        }
    }
    if (mu > 0) {
        for (int e = 0; e < n_edges; ++e) {
            const long a = edge_ij[2 * e], b = edge_ij[2 * e + 1];
            const double dx = p[2 * b] + edge_wrap[e] * offset - p[2 * a];
            const double dy = p[2 * a + 1] - p[2 * b + 1];
            double inv_len_sq = edge_l0[e];
            inv_len_sq = 1 / inv_len_sq / inv_len_sq;
            const double rh_x_sq = dx * dx * inv_len_sq;
            const double rh_y_sq = dy * dy * inv_len_sq;
            double m = mu * (1 - rh_x_sq);
            or_update(&s, a * 2, a * 2, m);
            or_update(&s, b * 2, b * 2, m);
            or_update(&s, a * 2, b * 2, -m);
            m = mu * (1 - rh_y_sq);
            or_update(&s, a * 2 + 1, a * 2 + 1, m);
            or_update(&s, b * 2 + 1, b * 2 + 1, m);
            or_update(&s, a * 2 + 1, b * 2 + 1, -m);
        }
    }
    qsort(s.c, (size_t)s.n, sizeof(or_contrib), or_contrib_cmp);
    long nnz = 0;
    for (long q = 0; q < s.n;) {
        double v = s.c[q].v;
        long r = q + 1;
        while (r < s.n && s.c[r].i == s.c[q].i && s.c[r].j == s.c[q].j) v += s.c[r++].v;
        if (fabs(v) > OR_SPR_TOL) {
            if (rows) {
                rows[nnz] = s.c[q].i;
                cols[nnz] = s.c[q].j;
                vals[nnz] = v;
            }
            nnz++;
        }
        q = r;
    }
    free(s.c);
    return nnz;
}

/* get_stretch_shear_energy (SPR:49-71) and get_bending_energy (:74-96) on
 * the full displacement field u (2N), summed in index order as the
 * reference sums them.  e_ss is computed when ks > 0 or mu > 0, e_bend when
 * kb > 0; otherwise 0 (the reference leaves them uninitialised). */
void or_spr_energies(const double *p, int n_edges, const int *edge_ij, const double *edge_l0,
                     const signed char *edge_wrap, double offset, double ks, double kb, double mu, int n_triples,
                     const int *tri_hjk, const signed char *tri_wrap, const double *u, double *e_ss_out,
                     double *e_bend_out) {
    double e_ss = 0, e_bend = 0;
    if (ks > 0 || mu > 0) {
        for (int e = 0; e < n_edges; ++e) {
            const int a = edge_ij[2 * e], b = edge_ij[2 * e + 1];
            const double length = edge_l0[e];
            const double dx = p[2 * b] + edge_wrap[e] * offset - p[2 * a];
            const double dy = p[2 * b + 1] - p[2 * a + 1];
            const double dux = u[b * 2] - u[a * 2];
            const double duy = u[b * 2 + 1] - u[a * 2 + 1];
            const double de = (dux * dx + duy * dy) / length;
            e_ss += .5 * ks * de * de;
            e_ss += .5 * mu * (dux * dux + duy * duy - de * de);
        }
    }
    if (kb > 0) {
        for (int t = 0; t < n_triples; ++t) {
            const int h = tri_hjk[3 * t], j = tri_hjk[3 * t + 1], k = tri_hjk[3 * t + 2];
            const double dx = p[2 * j] + offset * tri_wrap[2 * t] - p[2 * h];
            const double dy = p[2 * j + 1] - p[2 * h + 1];
            const double length_sq = dx * dx + dy * dy;
            const double dux = u[j * 2] + u[k * 2] - 2 * u[h * 2];
            const double duy = u[j * 2 + 1] + u[k * 2 + 1] - 2 * u[h * 2 + 1];
            const double du_c_r = dux * dy - duy * dx;
            e_bend += .5 * kb * du_c_r * du_c_r / length_sq;
        }
    }
    *e_ss_out = e_ss;
    *e_bend_out = e_bend;
}

/* affine_displacement (SPR:528-538) or add_displacement (:513-525) into
 * bc (2N): affine, every node (s (y - ymin), c (ymin - y)) with strains
 * c = compression / height, s = shear / height; otherwise the top nodes'
 * x = shear, y = -compression and every other entry left as it is. */
void or_spr_bc(int n_points, const double *p, double miny, double maxy, double compression, double shear, int affine,
               const unsigned char *is_top, double *bc) {
    if (affine) {
        const double c_strain = compression / (maxy - miny), s_strain = shear / (maxy - miny);
        for (int i = 0; i < n_points; ++i) {
            const double y = p[2 * i + 1];
            bc[i * 2] = s_strain * (y - miny);
            bc[i * 2 + 1] = c_strain * (miny - y);
        }
    } else {
        for (int i = 0; i < n_points; ++i)
            if (is_top[i]) {
                bc[i * 2 + 1] = -1 * compression;
                bc[i * 2] = 1 * shear;
            }
    }
}
