/*
 * nr_oracle.c — CPU restatement of large_strain_relax.cu's hot path.
 * TEST INFRASTRUCTURE ONLY (see nr_oracle.h).  Compile with
 * -ffp-contract=off; every fused multiply-add below is an explicit fma().
 */
#define _GNU_SOURCE
#include "nr_oracle.h"
#include "nr_oracle_internal.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Line reader with std::getline / istream::eof semantics.                   */
/* ------------------------------------------------------------------------ */

/* Reads the next line into r->buf (without '\n').  Sets r->eof when the end
 * of the file is reached before a '\n', as getline() on an ifstream does. */
const char *or_getline(or_lines *r) {
    ssize_t n = getline(&r->buf, &r->cap, r->f);
    if (n < 0) {
        r->eof = 1;
        if (r->buf) r->buf[0] = '\0';
        return r->buf ? r->buf : "";
    }
    if (n > 0 && r->buf[n - 1] == '\n') {
        r->buf[n - 1] = '\0';
    } else {
        r->eof = 1;
    }
    return r->buf;
}

/* large_strain_relax.cu:42-114 */
int or_read_network(const char *path, or_net *net) {
    memset(net, 0, sizeof(*net));
    or_lines r = {fopen(path, "r"), 0, NULL, 0};
    if (!r.f) return 0;
    int num_points = 0, num_edges = 0;
    double offset = 0;
    net->miny = FLT_MAX;
    net->maxy = FLT_MIN; /* the reference initialises max_y with FLT_MIN */
    const char *line = or_getline(&r);
    int num_read = sscanf(line, "%d %d %lf", &num_points, &num_edges, &offset);
    if (num_read < 3 || offset < 0 || num_points <= 0 || num_edges < 0) {
        fprintf(stderr, "Reading failed. The provided file has an invalid header.\n");
        fclose(r.f);
        free(r.buf);
        return 0;
    }
    net->offset = offset;
    net->points = (double *)malloc(sizeof(double) * 2 * (size_t)num_points);
    long np = 0;
    while (!r.eof && np < 2L * num_points) {
        double x, y;
        line = or_getline(&r);
        if (sscanf(line, "%lf %lf", &x, &y) == 2) {
            net->points[np++] = x;
            net->points[np++] = y;
            if (y < net->miny) net->miny = y;
            if (y > net->maxy) net->maxy = y;
        }
    }
    net->n_points = (int)(np / 2);
    if (r.eof) {
        fprintf(stderr, "Reading failed. Too few points were read.\n");
        fclose(r.f);
        free(r.buf);
        return 0;
    }
    net->edge_ij = (int *)malloc(sizeof(int) * 2 * (size_t)(num_edges + 1));
    net->edge_l0 = (double *)malloc(sizeof(double) * (size_t)(num_edges + 1));
    net->edge_wrap = (signed char *)malloc((size_t)(num_edges + 1));
    int ne = 0;
    while (!r.eof && ne < num_edges) {
        int i1, i2;
        signed char mult;
        line = or_getline(&r);
        if (sscanf(line, "%d %d %hhd\n", &i1, &i2, &mult) == 3) {
            int lo = i1 < i2 ? i1 : i2, hi = i1 < i2 ? i2 : i1;
            if (lo > -1 && hi < num_points) {
                double dx = net->points[2 * i2] + offset * mult - net->points[2 * i1];
                double dy = net->points[2 * i2 + 1] - net->points[2 * i1 + 1];
                net->edge_ij[2 * ne] = i1;
                net->edge_ij[2 * ne + 1] = i2;
                net->edge_l0[ne] = sqrt(dx * dx + dy * dy);
                net->edge_wrap[ne] = mult;
                ne++;
            } else {
                fprintf(stderr, "Reading failed due to an out-of-bounds point index.\n");
                net->n_edges = ne;
                fclose(r.f);
                free(r.buf);
                return 0;
            }
        }
    }
    net->n_edges = ne;
    fclose(r.f);
    free(r.buf);
    if (ne < num_edges) fprintf(stderr, "Too few edges were found.\n");
    return ne == num_edges;
}

/* large_strain_relax.cu:116-184.  Adjacency lists per node in edge order
 * (forward wrap for the first endpoint, negated for the second), hinges in
 * ascending node order, pairs (i<j) in list order, accepted when the two
 * arms are antiparallel to the absolute tolerance 1e-10 of :176. */
void or_get_triples(or_net *net) {
    free(net->tri_hjk);
    free(net->tri_wrap);
    const int n = net->n_points, ne = net->n_edges;
    int *deg = (int *)calloc((size_t)n + 1, sizeof(int));
    for (int e = 0; e < ne; ++e) {
        deg[net->edge_ij[2 * e]]++;
        deg[net->edge_ij[2 * e + 1]]++;
    }
    int *start = (int *)malloc(sizeof(int) * ((size_t)n + 1));
    start[0] = 0;
    for (int i = 0; i < n; ++i) start[i + 1] = start[i] + deg[i];
    int *fill = (int *)calloc((size_t)n, sizeof(int));
    int *nb = (int *)malloc(sizeof(int) * (size_t)(2 * ne + 1));
    signed char *nw = (signed char *)malloc((size_t)(2 * ne + 1));
    for (int e = 0; e < ne; ++e) {
        int a = net->edge_ij[2 * e], b = net->edge_ij[2 * e + 1];
        signed char w = net->edge_wrap[e];
        nb[start[a] + fill[a]] = b;
        nw[start[a] + fill[a]++] = w;
        nb[start[b] + fill[b]] = a;
        nw[start[b] + fill[b]++] = (signed char)(-w);
    }
    long cap = 16, nt = 0;
    int *hjk = (int *)malloc(sizeof(int) * 3 * cap);
    signed char *tw = (signed char *)malloc(2 * cap);
    const double *p = net->points;
    const double offset = net->offset;
    for (int h = 0; h < n; ++h) {
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
                if (dot < 0 && fabs(dot * dot - mag_sq) < 1e-10) {
                    if (nt == cap) {
                        cap *= 2;
                        hjk = (int *)realloc(hjk, sizeof(int) * 3 * cap);
                        tw = (signed char *)realloc(tw, 2 * cap);
                    }
                    hjk[3 * nt] = h;
                    hjk[3 * nt + 1] = j;
                    hjk[3 * nt + 2] = k;
                    tw[2 * nt] = nw[i];
                    tw[2 * nt + 1] = nw[k2];
                    nt++;
                }
            }
        }
    }
    net->tri_hjk = hjk;
    net->tri_wrap = tw;
    net->n_triples = (int)nt;
    free(deg);
    free(start);
    free(fill);
    free(nb);
    free(nw);
}

void or_free_net(or_net *net) {
    free(net->points);
    free(net->edge_ij);
    free(net->edge_l0);
    free(net->edge_wrap);
    free(net->tri_hjk);
    free(net->tri_wrap);
    memset(net, 0, sizeof(*net));
}

/* large_strain_relax.cu:895-901: rows within 1e-10 of the extreme y are
 * clamped (code 0); every other node is free in x and y (code 3). */
void or_fcodes(const or_net *net, const double *points, unsigned char *fcodes) {
    for (int i = 0; i < net->n_points; ++i) {
        const double y = points[2 * i + 1];
        fcodes[i] = (y < net->miny + 1e-10 || y > net->maxy - 1e-10) ? 0 : 3;
    }
}

/* large_strain_relax.cu:527-537 over the n_points nodes only (the reference
 * launches 2N threads and also touches the N entries past the array). */
void or_affine_displace(int n_points, double *pos, double miny, double yrange, double xdisp, double ydisp) {
    for (int i = 0; i < n_points; ++i) {
        pos[2 * i] += xdisp * (pos[2 * i + 1] - miny) / yrange;
        pos[2 * i + 1] += ydisp * (pos[2 * i + 1] - miny) / yrange;
    }
}

/* ------------------------------------------------------------------------ */
/* Canonical math                                                            */
/* ------------------------------------------------------------------------ */

/* Polynomial of atan(u) = u + u*z*Q(z), z = u^2, |u| <= tan(pi/8); derived by
 * network_relaxation_gb300/csrc/gen_atan_coeffs.py (Chebyshev interpolation
 * in 60-digit arithmetic).  Highest power first. */
static const double OR_ATAN_Q[11] = {
    -0.01917688711906226, 0.03923165829558719, -0.0508544973794026, 0.0585814891280221,
    -0.06664511447381948, 0.07692183190826087, -0.09090904578123903, 0.11111111015256361,
    -0.14285714284666542, 0.1999999999999552, -0.3333333333333333,
};
#define OR_TAN_PI_8 0.41421356237309503
#define OR_PIO4_HI 0.7853981633974483
#define OR_PIO4_LO 3.061616997868383e-17
#define OR_PIO2_HI 1.5707963267948966
#define OR_PIO2_LO 6.123233995736766e-17
#define OR_PI_HI 3.141592653589793
#define OR_PI_LO 1.2246467991473532e-16

/* atan2 built from +, -, *, /, fma only (identical bits on any IEEE machine).
 * Quadrant / octant reduction, atan(t) = pi/4 + atan((t-1)/(t+1)) above
 * tan(pi/8), then the polynomial.  For finite non-zero arguments it agrees
 * with atan2 to about one ulp; atan2(0, 0) = 0. */
double or_atan2(double y, double x) {
    const double ax = fabs(x), ay = fabs(y);
    const int swap = ay > ax;
    const double num = swap ? ax : ay;
    const double den = swap ? ay : ax;
    const double t = den == 0.0 ? 0.0 : num / den;
    const int red = t > OR_TAN_PI_8;
    const double u = red ? (t - 1.0) / (t + 1.0) : t;
    const double z = u * u;
    double q = OR_ATAN_Q[0];
    for (int i = 1; i < 11; ++i) q = fma(q, z, OR_ATAN_Q[i]);
    double r = fma(u * z, q, u);
    if (red) r = OR_PIO4_HI + (OR_PIO4_LO + r);
    if (swap) r = OR_PIO2_HI + (OR_PIO2_LO - r);
    if (x < 0.0) r = OR_PI_HI + (OR_PI_LO - r);
    return y < 0.0 ? -r : r;
}

/* Butterfly over 32 lanes (xor offsets 16, 8, 4, 2, 1), as a warp shuffle
 * reduction computes it; returns lane 0's (= every lane's) value. */
static double or_butterfly32(double *a) {
    for (int off = 16; off >= 1; off >>= 1)
        for (int i = 0; i < off; ++i) a[i] = a[i] + a[i + off];
    return a[0];
}

static double or_tree8(const double *w) {
    return ((w[0] + w[1]) + (w[2] + w[3])) + ((w[4] + w[5]) + (w[6] + w[7]));
}

/* Sum of 256 lanes: butterfly within each warp of 32, then the 8 warp sums
 * pairwise. */
static double or_block256(const double *lanes) {
    double tmp[32], w[8];
    for (int g = 0; g < 8; ++g) {
        memcpy(tmp, lanes + 32 * g, sizeof(tmp));
        w[g] = or_butterfly32(tmp);
    }
    return or_tree8(w);
}

/* The fixed summation order that replaces cublasDasum (large_strain_relax.cu:743, :751) and the
 * cuBLAS dot / nrm2 reductions of run_fire_md, whose order is unspecified.
 * Canonical reduction: terms are grouped in tiles of 256 consecutive items
 * (missing items are 0); each tile is reduced by or_block256; tile sums are
 * accumulated per lane (lane k sums tiles k, k+256, ... in order, starting
 * from tile k) and the 256 lane sums are reduced by or_block256. */
double or_canon_sum(const double *terms, long n) {
    const long T = (n + 255) / 256;
    double lanes[256];
    double acc[256];
    for (int k = 0; k < 256; ++k) acc[k] = 0.0;
    for (long t = 0; t < T; ++t) {
        for (int k = 0; k < 256; ++k) {
            const long i = 256 * t + k;
            lanes[k] = i < n ? terms[i] : 0.0;
        }
        const double s = or_block256(lanes);
        if (t < 256) acc[t] = s;
        else acc[t % 256] = acc[t % 256] + s;
    }
    return or_block256(acc);
}

/* ------------------------------------------------------------------------ */
/* Forces and energies                                                       */
/* ------------------------------------------------------------------------ */

/* large_strain_relax.cu:386-414 (stretch) then :417-469 (bending), each
 * contribution masked by the node's fcode bits, summed per node in index
 * order.  Skipped entirely when ks <= 0 / kb <= 0 (:629, :634). */
void or_forces(const or_model *m, const double *pos, double *F) {
    const double W = m->width;
    memset(F, 0, sizeof(double) * 2 * (size_t)m->n_points);
    if (m->ks > 0) {
        for (int b = 0; b < m->n_edges; ++b) {
            const int i1 = m->edge_ij[2 * b], i2 = m->edge_ij[2 * b + 1];
            const double k = m->bond_k ? m->bond_k[b] : m->ks;
            const double l0 = m->edge_l0[b];
            const double wW = (double)m->edge_wrap[b] * W;
            const double x1 = pos[2 * i1], y1 = pos[2 * i1 + 1];
            const double x2 = pos[2 * i2], y2 = pos[2 * i2 + 1];
            const double rx = (x1 - x2) - wW, ry = y1 - y2;
            const double inv = 1.0 / sqrt(fma(rx, rx, ry * ry));
            const double s = k * fma(-l0, inv, 1.0);
            const double fx = s * ((x2 + wW) - x1);
            const double fy = s * (y2 - y1);
            const unsigned char c1 = m->fcodes[i1], c2 = m->fcodes[i2];
            F[2 * i1] = F[2 * i1] + fx * (double)(c1 & 1);
            F[2 * i1 + 1] = F[2 * i1 + 1] + fy * (double)((c1 & 2) >> 1);
            F[2 * i2] = F[2 * i2] + (-fx) * (double)(c2 & 1);
            F[2 * i2 + 1] = F[2 * i2 + 1] + (-fy) * (double)((c2 & 2) >> 1);
        }
    }
    if (m->kb > 0) {
        for (int t = 0; t < m->n_triples; ++t) {
            const int h = m->tri_hjk[3 * t], j = m->tri_hjk[3 * t + 1], k = m->tri_hjk[3 * t + 2];
            const double kb = m->tri_kb ? m->tri_kb[t] : m->kb;
            const double phi0 = m->tri_phi0 ? m->tri_phi0[t] : 0.0;
            const double wj = (double)m->tri_wrap[2 * t] * W, wk = (double)m->tri_wrap[2 * t + 1] * W;
            const double xh = pos[2 * h], yh = pos[2 * h + 1];
            const double ax = (pos[2 * j] + wj) - xh, ay = pos[2 * j + 1] - yh;
            const double bx = (pos[2 * k] + wk) - xh, by = pos[2 * k + 1] - yh;
            const double c = fma(ax, by, -(ay * bx));
            const double d = fma(ax, bx, ay * by);
            const double dth = or_atan2(-c, -d) - phi0;
            const double g = kb * dth;
            const double g2 = g / fma(ax, ax, ay * ay);
            const double g3 = g / fma(bx, bx, by * by);
            const double fjx = -ay * g2, fjy = ax * g2;
            const double fkx = by * g3, fky = -bx * g3;
            const double fhx = -fjx - fkx, fhy = -fjy - fky;
            const unsigned char ch = m->fcodes[h], cj = m->fcodes[j], ck = m->fcodes[k];
            F[2 * h] = F[2 * h] + fhx * (double)(ch & 1);
            F[2 * h + 1] = F[2 * h + 1] + fhy * (double)((ch & 2) >> 1);
            F[2 * j] = F[2 * j] + fjx * (double)(cj & 1);
            F[2 * j + 1] = F[2 * j + 1] + fjy * (double)((cj & 2) >> 1);
            F[2 * k] = F[2 * k] + fkx * (double)(ck & 1);
            F[2 * k + 1] = F[2 * k + 1] + fky * (double)((ck & 2) >> 1);
        }
    }
    if (m->bmod > 0) or_gel_forces(m, pos, F);
}

/* large_strain_relax.cu:472-490 and :493-523, each summed with the
 * canonical reduction in place of cublasDasum (:743, :751). */
void or_energies(const or_model *m, const double *pos, double *e_stretch, double *e_bend) {
    const double W = m->width;
    *e_stretch = 0.0;
    *e_bend = 0.0;
    if (m->ks > 0 && m->n_edges > 0) {
        double *terms = (double *)malloc(sizeof(double) * (size_t)m->n_edges);
        for (int b = 0; b < m->n_edges; ++b) {
            const int i1 = m->edge_ij[2 * b], i2 = m->edge_ij[2 * b + 1];
            const double k = m->bond_k ? m->bond_k[b] : m->ks;
            const double wW = (double)m->edge_wrap[b] * W;
            const double rx = (pos[2 * i1] - pos[2 * i2]) - wW, ry = pos[2 * i1 + 1] - pos[2 * i2 + 1];
            const double dd = sqrt(fma(rx, rx, ry * ry)) - m->edge_l0[b];
            terms[b] = ((0.5 * k) * dd) * dd;
        }
        *e_stretch = or_canon_sum(terms, m->n_edges);
        free(terms);
    }
    if (m->kb > 0 && m->n_triples > 0) {
        double *terms = (double *)malloc(sizeof(double) * (size_t)m->n_triples);
        for (int t = 0; t < m->n_triples; ++t) {
            const int h = m->tri_hjk[3 * t], j = m->tri_hjk[3 * t + 1], k = m->tri_hjk[3 * t + 2];
            const double kb = m->tri_kb ? m->tri_kb[t] : m->kb;
            const double phi0 = m->tri_phi0 ? m->tri_phi0[t] : 0.0;
            const double wj = (double)m->tri_wrap[2 * t] * W, wk = (double)m->tri_wrap[2 * t + 1] * W;
            const double xh = pos[2 * h], yh = pos[2 * h + 1];
            const double ax = (pos[2 * j] + wj) - xh, ay = pos[2 * j + 1] - yh;
            const double bx = (pos[2 * k] + wk) - xh, by = pos[2 * k + 1] - yh;
            const double c = fma(ax, by, -(ay * bx));
            const double d = fma(ax, bx, ay * by);
            const double dth = or_atan2(-c, -d) - phi0;
            terms[t] = ((0.5 * kb) * dth) * dth;
        }
        *e_bend = or_canon_sum(terms, m->n_triples);
        free(terms);
    }
}

/* Virial W = -sum_n r_n (x) F_n of the stretch and bending forces (no
 * counterpart in the reference, which reports no stress; the library's
 * stress output).  Per bond, with r = r_j - r_i (minimum image) and f the
 * stretch force on i of large_strain_relax.cu:386-414: W_ab = r_a f_b.  Per
 * triple, with arms a = r_hj, b = r_hk and the bending forces F_j, F_k of
 * :417-469: W_ab = -(a_a F_j,b + b_a F_k,b).  Each component is summed over
 * bonds and over triples separately with or_canon_sum, the two sums added:
 * w = {W_xx, W_yy, W_xy}.  sigma = W / area; W_xy = dE/dgamma under the
 * affine shear of :527-537. */
void or_virial(const or_model *m, const double *pos, double w[3]) {
    const double W = m->width;
    double wb[3] = {0.0, 0.0, 0.0}, wt[3] = {0.0, 0.0, 0.0};
    if (m->ks > 0 && m->n_edges > 0) {
        double *terms = (double *)malloc(sizeof(double) * 3 * (size_t)m->n_edges);
        for (int b = 0; b < m->n_edges; ++b) {
            const int i1 = m->edge_ij[2 * b], i2 = m->edge_ij[2 * b + 1];
            const double k = m->bond_k ? m->bond_k[b] : m->ks;
            const double l0 = m->edge_l0[b];
            const double wW = (double)m->edge_wrap[b] * W;
            const double x1 = pos[2 * i1], y1 = pos[2 * i1 + 1];
            const double x2 = pos[2 * i2], y2 = pos[2 * i2 + 1];
            const double rx0 = (x1 - x2) - wW, ry0 = y1 - y2;
            const double inv = 1.0 / sqrt(fma(rx0, rx0, ry0 * ry0));
            const double sc = k * fma(-l0, inv, 1.0);
            const double fx = sc * ((x2 + wW) - x1);
            const double fy = sc * (y2 - y1);
            const double rx = (x2 + wW) - x1, ry = y2 - y1;
            terms[b] = rx * fx;
            terms[m->n_edges + b] = ry * fy;
            terms[2 * (size_t)m->n_edges + b] = ry * fx;
        }
        for (int c = 0; c < 3; ++c) wb[c] = or_canon_sum(terms + (size_t)c * m->n_edges, m->n_edges);
        free(terms);
    }
    if (m->kb > 0 && m->n_triples > 0) {
        double *terms = (double *)malloc(sizeof(double) * 3 * (size_t)m->n_triples);
        for (int t = 0; t < m->n_triples; ++t) {
            const int h = m->tri_hjk[3 * t], j = m->tri_hjk[3 * t + 1], k = m->tri_hjk[3 * t + 2];
            const double kb = m->tri_kb ? m->tri_kb[t] : m->kb;
            const double phi0 = m->tri_phi0 ? m->tri_phi0[t] : 0.0;
            const double wj = (double)m->tri_wrap[2 * t] * W, wk = (double)m->tri_wrap[2 * t + 1] * W;
            const double xh = pos[2 * h], yh = pos[2 * h + 1];
            const double ax = (pos[2 * j] + wj) - xh, ay = pos[2 * j + 1] - yh;
            const double bx = (pos[2 * k] + wk) - xh, by = pos[2 * k + 1] - yh;
            const double c = fma(ax, by, -(ay * bx));
            const double d = fma(ax, bx, ay * by);
            const double g = kb * (or_atan2(-c, -d) - phi0);
            const double g2 = g / fma(ax, ax, ay * ay);
            const double g3 = g / fma(bx, bx, by * by);
            const double fjx = -ay * g2, fjy = ax * g2, fkx = by * g3, fky = -bx * g3;
            terms[t] = -fma(ax, fjx, bx * fkx);
            terms[m->n_triples + t] = -fma(ay, fjy, by * fky);
            terms[2 * (size_t)m->n_triples + t] = -fma(ay, fjx, by * fkx);
        }
        for (int c = 0; c < 3; ++c) wt[c] = or_canon_sum(terms + (size_t)c * m->n_triples, m->n_triples);
        free(terms);
    }
    for (int c = 0; c < 3; ++c) w[c] = wb[c] + wt[c];
}

/* ------------------------------------------------------------------------ */
/* FIRE (large_strain_relax.cu:596-762)                                      */
/* ------------------------------------------------------------------------ */

typedef struct {
    double P, V2, F2, maxF2;
} or_sums;

static or_sums or_fire_sums(int n, const double *v, const double *F, double *scratch) {
    or_sums s;
    double *t = scratch;
    for (int i = 0; i < n; ++i) t[i] = fma(v[2 * i], F[2 * i], v[2 * i + 1] * F[2 * i + 1]);
    s.P = or_canon_sum(t, n);
    for (int i = 0; i < n; ++i) t[i] = fma(v[2 * i], v[2 * i], v[2 * i + 1] * v[2 * i + 1]);
    s.V2 = or_canon_sum(t, n);
    s.maxF2 = 0.0;
    for (int i = 0; i < n; ++i) {
        t[i] = fma(F[2 * i], F[2 * i], F[2 * i + 1] * F[2 * i + 1]);
        if (t[i] > s.maxF2) s.maxF2 = t[i];
    }
    s.F2 = or_canon_sum(t, n);
    return s;
}

/* run_fire_md, large_strain_relax.cu:596-762: FIRE from v = 0 and dt = dt_max, velocity-Verlet drift and
 * kicks (:655-677), P = F.v and mixing (:686-691), dt / alpha adaption (:694-713), the stop test (:716,
 * RMS or max criterion), energies after the loop (:723-751); reductions by or_canon_sum. */
int or_fire(const or_model *m, double *x, double *v, double *F, const or_fire_params *p, or_report *rep) {
    const int n = m->n_points;
    const long ndof = 2L * n;
    double *scratch = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    const double alpha_start = p->alpha0, falpha = p->falpha, dt_max = p->dt_max, finc = p->finc,
                 fdec = p->fdec, mass = p->mass;
    double alpha = alpha_start;
    double dt = dt_max;
    double dt_sq_mult = .5 * dt * dt / mass;
    double dt_mult = .5 * dt / mass;
    const double sqrt_dof = sqrt((double)ndof);
    int since_leq_0 = 0, step = 0;

    memset(v, 0, sizeof(double) * ndof);
    or_forces(m, x, F);
    or_sums s = or_fire_sums(n, v, F, scratch);
    double fmag = sqrt(s.F2);
    double maxf = sqrt(s.maxF2);
    int converged = 0;

    while (step < p->max_steps) {
        step++;
        for (long i = 0; i < ndof; ++i) {
            x[i] = fma(dt, v[i], x[i]);
            x[i] = fma(dt_sq_mult, F[i], x[i]);
            v[i] = fma(dt_mult, F[i], v[i]);
        }
        or_forces(m, x, F);
        for (long i = 0; i < ndof; ++i) v[i] = fma(dt_mult, F[i], v[i]);
        s = or_fire_sums(n, v, F, scratch);
        const double power = s.P;
        const double vmag = sqrt(s.V2);
        fmag = sqrt(s.F2);
        maxf = sqrt(s.maxF2);
        const double a_vm_o_fm = alpha * vmag / fmag;
        const double neg_alpha = -alpha;
        for (long i = 0; i < ndof; ++i) {
            v[i] = fma(neg_alpha, v[i], v[i]);
            v[i] = fma(a_vm_o_fm, F[i], v[i]);
        }
        if (power > 0) {
            since_leq_0++;
            if (since_leq_0 > p->nmin) {
                dt = fmin(dt * finc, dt_max);
                dt_mult = .5 * dt / mass;
                dt_sq_mult = .5 * dt * dt / mass;
                alpha *= falpha;
            }
        } else {
            since_leq_0 = 0;
            dt *= fdec;
            dt_mult = .5 * dt / mass;
            dt_sq_mult = dt * dt * .5 / mass;
            alpha = alpha_start;
            memset(v, 0, sizeof(double) * ndof);
        }
        const int done = p->criterion == OR_CRIT_MAX ? (maxf < p->fcut) : (fmag / sqrt_dof < p->fcut);
        if (done) {
            converged = 1;
            break;
        }
    }
    if (!converged) {
        converged = p->criterion == OR_CRIT_MAX ? (maxf < p->fcut) : (fmag / sqrt_dof < p->fcut);
    }
    rep->rms_force = fmag / sqrt_dof;
    rep->max_force = maxf;
    rep->steps = step;
    rep->converged = converged;
    or_energies(m, x, &rep->e_stretch, &rep->e_bend);
    rep->e_gel = m->bmod > 0 ? or_gel_energy(m, x) : 0.0;
    free(scratch);
    return converged;
}

/* ------------------------------------------------------------------------ */
/* Strain protocol (large_strain_relax.cu:917-999, strain mode)              */
/* ------------------------------------------------------------------------ */

int or_sweep(const or_model *m, double *pos, double miny, double yrange, const or_fire_params *p,
             const double compr[3], const double shear[3], double *records, int max_records,
             double *shear_pos) {
    const int n = m->n_points;
    double *v = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    double *F = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    const double smult = yrange;
    int nrec = 0;
    or_report rep;
    double min_disp = compr[0] * smult, max_disp = compr[1] * smult, inc = compr[2] * smult;
    double curr_disp = 0.0;
    if (max_disp > 0) {
        for (curr_disp = min_disp; curr_disp <= max_disp + 1e-10; curr_disp += inc) {
            or_affine_displace(n, pos, miny, yrange, 0, -inc);
            or_fire(m, pos, v, F, p, &rep);
            if (nrec < max_records) {
                double *r = records + 8 * nrec;
                r[0] = 0.0; r[1] = curr_disp; r[2] = rep.e_stretch; r[3] = rep.e_bend;
                r[4] = rep.rms_force; r[5] = rep.max_force; r[6] = rep.steps; r[7] = 0;
                nrec++;
            }
            if (inc <= 0) break; /* the reference loops forever on inc == 0 */
        }
    }
    const double max_comp = max_disp > min_disp ? curr_disp - inc : max_disp;
    min_disp = shear[0] * smult;
    max_disp = shear[1] * smult;
    inc = shear[2] * smult;
    if (max_disp > 0) {
        for (curr_disp = min_disp; curr_disp <= max_disp + 1e-10; curr_disp += inc) {
            or_affine_displace(n, pos, miny, yrange, inc, 0);
            or_fire(m, pos, v, F, p, &rep);
            if (nrec < max_records) {
                double *r = records + 8 * nrec;
                r[0] = curr_disp; r[1] = max_comp; r[2] = rep.e_stretch; r[3] = rep.e_bend;
                r[4] = rep.rms_force; r[5] = rep.max_force; r[6] = rep.steps; r[7] = 1;
                if (shear_pos) memcpy(shear_pos + 2 * (size_t)n * nrec, pos, sizeof(double) * 2 * (size_t)n);
                nrec++;
            }
            if (inc <= 0) break;
        }
    }
    free(v);
    free(F);
    return nrec;
}

/* ------------------------------------------------------------------------ */
/* Batch over host threads                                                   */
/* ------------------------------------------------------------------------ */

typedef struct {
    int n;
    const or_model *models;
    double **pos;
    const or_fire_params *params;
    or_report *reps;
    int next;
    pthread_mutex_t lock;
} or_batch_job;

static void *or_batch_worker(void *arg) {
    or_batch_job *job = (or_batch_job *)arg;
    for (;;) {
        pthread_mutex_lock(&job->lock);
        const int i = job->next++;
        pthread_mutex_unlock(&job->lock);
        if (i >= job->n) break;
        const int np = job->models[i].n_points;
        double *v = (double *)malloc(sizeof(double) * 2 * (size_t)np);
        double *F = (double *)malloc(sizeof(double) * 2 * (size_t)np);
        or_fire(&job->models[i], job->pos[i], v, F, &job->params[i], &job->reps[i]);
        free(v);
        free(F);
    }
    return NULL;
}

/* or_fire over n independent networks on n_threads host threads (the CPU baseline of batches; the
 * reference relaxes its file list one network at a time, large_strain_relax.cu:1040-1042). */
void or_fire_batch(int n, const or_model *models, double **pos, const or_fire_params *params, or_report *reps,
                   int n_threads) {
    or_batch_job job = {n, models, pos, params, reps, 0, PTHREAD_MUTEX_INITIALIZER};
    if (n_threads < 1) n_threads = 1;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n_threads);
    for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, or_batch_worker, &job);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    free(th);
}

/* ----- post-relaxation analyses (strain_calc, axial_contribution, na_calc) ----- */

/* strain_calc.cpp:96-120: the engineering strain of every bond under a displacement field. */
void or_bond_strains(int n_edges, const int *edge_ij, const signed char *wrap, double width, const double *pos0,
                     const double *disp, double *strains) {
    for (int b = 0; b < n_edges; ++b) {
        const int i1 = edge_ij[2 * b], i2 = edge_ij[2 * b + 1];
        /* strain_calc.cpp:108-116, operation for operation */
        const double dxi = pos0[2 * i2] + wrap[b] * width - pos0[2 * i1];
        const double dyi = pos0[2 * i2 + 1] - pos0[2 * i1 + 1];
        const double dxf = dxi + disp[2 * i2] - disp[2 * i1];
        const double dyf = dyi + disp[2 * i2 + 1] - disp[2 * i1 + 1];
        const double li = sqrt(dxi * dxi + dyi * dyi);
        const double lf = sqrt(dxf * dxf + dyf * dyf);
        strains[b] = (lf - li) / li;
    }
}

/* axial_contribution.cpp:64-70, 176-190: the linearised stretch energy of a displacement field
 * (summed by or_canon_sum). */
double or_linear_axial_energy(int n_edges, const int *edge_ij, const signed char *wrap, double width, double k,
                              const double *pos0, const double *disp) {
    double *terms = (double *)malloc(sizeof(double) * (size_t)(n_edges > 0 ? n_edges : 1));
    for (int b = 0; b < n_edges; ++b) {
        const int i1 = edge_ij[2 * b], i2 = edge_ij[2 * b + 1];
        /* axial_contribution.cpp:64-70 */
        double dx = pos0[2 * i2] + width * wrap[b] - pos0[2 * i1];
        double dy = pos0[2 * i2 + 1] - pos0[2 * i1 + 1];
        const double length = sqrt(dx * dx + dy * dy);
        dx /= length;
        dy /= length;
        /* axial_contribution.cpp:178-188 */
        const double proj = (disp[2 * i2] - disp[2 * i1]) * dx + (disp[2 * i2 + 1] - disp[2 * i1 + 1]) * dy;
        terms[b] = .5 * proj * proj;
    }
    const double e = or_canon_sum(terms, n_edges);
    free(terms);
    return e * k;
}

/* calc_na_val, na_calc.cpp:308-327: the mean squared deviation from the affine field (summed by
 * or_canon_sum; the reference sums in node order). */
double or_nonaffinity(int n_points, const double *pos0, const double *disp, double miny, double axial_strain,
                      double shear_strain) {
    double *terms = (double *)malloc(sizeof(double) * (size_t)(n_points > 0 ? n_points : 1));
    for (int i = 0; i < n_points; ++i) {
        /* na_calc.cpp:313-322 */
        const double y = pos0[2 * i + 1];
        const double ux_a = disp[2 * i], uy_a = disp[2 * i + 1];
        const double ux_e = (y - miny) * shear_strain, uy_e = (y - miny) * axial_strain;
        terms[i] = (ux_a - ux_e) * (ux_a - ux_e) + (uy_a - uy_e) * (uy_a - uy_e);
    }
    const double na = or_canon_sum(terms, n_points);
    free(terms);
    return na / n_points;
}
