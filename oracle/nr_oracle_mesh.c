/*
 * nr_oracle_mesh.c — CPU restatement of the gel coupling of
 * network_mesh_relax.cu (network + FEM gel composites).
 * TEST INFRASTRUCTURE ONLY (see nr_oracle.h).  Compile with
 * -ffp-contract=off.
 *
 * The gel arithmetic keeps the reference's expressions and association
 * (plain multiplies and adds, no fused operations), so on a host compiled
 * without FMA contraction the element forces equal the reference's
 * gel_forces term by term; per node they are added in element index order,
 * x then y, first the dU/dF_i1 term then the dU/dF_i2 term, which is the
 * reference's atomicAdd sequence serialised in element order.
 */
#define _GNU_SOURCE
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nr_oracle.h"
#include "nr_oracle_internal.h"

#define OR_FLT_TOL 1e-10

/* PointComp (network_mesh_relax.cu:53-61): x first with tolerance, then y. */
static int or_point_less(double ax, double ay, double bx, double by) {
    if (ax < bx - OR_FLT_TOL) return 1;
    if (ax > bx + OR_FLT_TOL) return 0;
    return ay < by - OR_FLT_TOL;
}

/* First position in keys[0..n) whose point is not less than (x, y). */
static int or_lower_bound(const int *keys, int n, const double *pts, double x, double y) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (or_point_less(pts[2 * keys[mid]], pts[2 * keys[mid] + 1], x, y)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

/* :219-227.  The std::map<Point, int, PointComp> of the reader is a sorted
 * array of point indices: points are inserted in file order and a point
 * equivalent to one already present is not inserted (map::insert keeps the
 * first).  Left-edge points (x < minx + 1e-10) are visited in map order and
 * paired with the point found at (x + offset, y). */
int or_mesh_pairs(int n_points, const double *pts, double offset, double minx, int *pairs) {
    int *keys = (int *)malloc(sizeof(int) * (size_t)(n_points > 0 ? n_points : 1));
    int nk = 0, np = 0;
    for (int i = 0; i < n_points; ++i) {
        const double x = pts[2 * i], y = pts[2 * i + 1];
        const int pos = or_lower_bound(keys, nk, pts, x, y);
        if (pos < nk && !or_point_less(x, y, pts[2 * keys[pos]], pts[2 * keys[pos] + 1])) continue;
        memmove(keys + pos + 1, keys + pos, sizeof(int) * (size_t)(nk - pos));
        keys[pos] = i;
        nk++;
    }
    for (int k = 0; k < nk && pts[2 * keys[k]] < minx + OR_FLT_TOL; ++k) {
        const double tx = pts[2 * keys[k]] + offset, ty = pts[2 * keys[k] + 1];
        const int pos = or_lower_bound(keys, nk, pts, tx, ty);
        if (pos < nk && !or_point_less(tx, ty, pts[2 * keys[pos]], pts[2 * keys[pos] + 1])) {
            pairs[2 * np] = keys[k];
            pairs[2 * np + 1] = keys[pos];
            np++;
        }
    }
    free(keys);
    return np;
}

static int or_mesh_fail(or_lines *r, const char *msg) {
    fprintf(stderr, "%s", msg);
    if (r->f) fclose(r->f);
    free(r->buf);
    r->f = NULL;
    r->buf = NULL;
    return 0;
}

/* network_mesh_relax.cu:72-230 */
int or_read_network_mesh(const char *path, or_mesh *mesh) {
    memset(mesh, 0, sizeof(*mesh));
    or_net *net = &mesh->net;
    or_lines r = {fopen(path, "r"), 0, NULL, 0};
    if (!r.f) return 0;
    int num_points = 0, num_edges = 0, num_facets = 0;
    double offset = 0;
    mesh->minx = FLT_MAX;
    net->miny = FLT_MAX;
    mesh->maxx = FLT_MIN; /* the reference initialises the maxima with FLT_MIN */
    net->maxy = FLT_MIN;
    const char *line = or_getline(&r);
    const int num_read = sscanf(line, "%d %d %d %lf", &num_points, &num_edges, &num_facets, &offset);
    if (num_read < 4 || offset < 0 || num_points <= 0 || num_edges < 0 || num_facets < 0)
        return or_mesh_fail(&r, "Reading failed. The provided file has an invalid header.\n");
    net->offset = offset;
    net->points = (double *)malloc(sizeof(double) * 2 * (size_t)num_points);
    long np = 0;
    while (!r.eof && np < 2L * num_points) {
        double x, y;
        line = or_getline(&r);
        if (sscanf(line, "%lf %lf", &x, &y) == 2) {
            net->points[np++] = x;
            net->points[np++] = y;
            if (x < mesh->minx) mesh->minx = x;
            if (y < net->miny) net->miny = y;
            if (x > mesh->maxx) mesh->maxx = x;
            if (y > net->maxy) net->maxy = y;
        }
    }
    net->n_points = (int)(np / 2);
    if (r.eof) return or_mesh_fail(&r, "Reading failed. Too few points were read.\n");
    net->edge_ij = (int *)malloc(sizeof(int) * 2 * (size_t)(num_edges + 1));
    net->edge_l0 = (double *)malloc(sizeof(double) * (size_t)(num_edges + 1));
    net->edge_wrap = (signed char *)malloc((size_t)(num_edges + 1));
    int ne = 0;
    while (!r.eof && ne < num_edges) {
        int i1, i2;
        signed char mult;
        line = or_getline(&r);
        if (sscanf(line, "%d %d %hhd\n", &i1, &i2, &mult) == 3) {
            const int lo = i1 < i2 ? i1 : i2, hi = i1 < i2 ? i2 : i1;
            if (lo > -1 && hi < num_points) {
                const double dx = net->points[2 * i2] + offset * mult - net->points[2 * i1];
                const double dy = net->points[2 * i2 + 1] - net->points[2 * i1 + 1];
                net->edge_ij[2 * ne] = i1;
                net->edge_ij[2 * ne + 1] = i2;
                net->edge_l0[ne] = sqrt(dx * dx + dy * dy);
                net->edge_wrap[ne] = mult;
                ne++;
            } else {
                net->n_edges = ne;
                return or_mesh_fail(&r, "Reading failed due to an out-of-bounds point index.\n");
            }
        }
    }
    net->n_edges = ne;
    if (ne < num_edges) return or_mesh_fail(&r, "Too few edges were read.\n");
    if (r.eof && num_facets > 0) return or_mesh_fail(&r, "The file ended before facets could be read.\n");
    mesh->facets = (int *)malloc(sizeof(int) * 3 * (size_t)(num_facets + 1));
    int nf = 0;
    while (!r.eof && nf < num_facets) {
        int i1, i2, i3;
        line = or_getline(&r);
        if (sscanf(line, "%d %d %d\n", &i1, &i2, &i3) == 3) {
            if (i1 >= 0 && i1 <= num_points - 1 && i2 >= 0 && i2 <= num_points - 1 && i3 >= 0 &&
                i3 <= num_points - 1) {
                mesh->facets[3 * nf] = i1;
                mesh->facets[3 * nf + 1] = i2;
                mesh->facets[3 * nf + 2] = i3;
                nf++;
            } else {
                mesh->n_facets = nf;
                return or_mesh_fail(&r, "Reading failed due to an out-of-bounds point index.\n");
            }
        }
    }
    mesh->n_facets = nf;
    if (nf < num_facets) return or_mesh_fail(&r, "Too few facets were read.\n");
    if (r.eof && num_facets > 0) return or_mesh_fail(&r, "The file ended before facets could be read.\n");
    mesh->areas = (double *)malloc(sizeof(double) * (size_t)(num_facets + 1));
    while (!r.eof && mesh->n_areas < num_facets) {
        double area;
        line = or_getline(&r);
        if (sscanf(line, "%lf", &area) == 1) {
            if (area > 0) mesh->areas[mesh->n_areas++] = area;
            else return or_mesh_fail(&r, "An illegal area was specified.\n");
        }
    }
    fclose(r.f);
    free(r.buf);
    if (mesh->n_areas < num_facets) {
        fprintf(stderr, "Too few areas were specified.\n");
        return 0;
    }
    mesh->mpairs = (int *)malloc(sizeof(int) * 2 * (size_t)(net->n_points > 0 ? net->n_points : 1));
    mesh->n_mpairs = or_mesh_pairs(net->n_points, net->points, offset, mesh->minx, mesh->mpairs);
    return 1;
}

void or_free_mesh(or_mesh *mesh) {
    or_free_net(&mesh->net);
    free(mesh->facets);
    free(mesh->areas);
    free(mesh->mpairs);
    memset(mesh, 0, sizeof(*mesh));
}

/* :503-531 */
void or_inv_mats(int n_elems, const double *pos, const int *el, double *inv) {
    for (int e = 0; e < n_elems; ++e) {
        const int i1 = el[3 * e], i2 = el[3 * e + 1], i3 = el[3 * e + 2];
        const double x1 = pos[2 * i1], y1 = pos[2 * i1 + 1];
        const double x2 = pos[2 * i2], y2 = pos[2 * i2 + 1];
        const double x3 = pos[2 * i3], y3 = pos[2 * i3 + 1];
        const double det = x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2);
        inv[6 * e] = (y2 - y3) / det;
        inv[6 * e + 1] = (x3 - x2) / det;
        inv[6 * e + 2] = (y3 - y1) / det;
        inv[6 * e + 3] = (x1 - x3) / det;
        inv[6 * e + 4] = (y1 - y2) / det;
        inv[6 * e + 5] = (x2 - x1) / det;
    }
}

/* :796-806 over the n_points nodes (the reference launches 2N threads and
 * also scales the N entries past the array). */
void or_dilate(int n_points, double *pos, double minx, double miny, double factor) {
    for (int i = 0; i < n_points; ++i) {
        pos[2 * i] = minx + factor * (pos[2 * i] - minx);
        pos[2 * i + 1] = miny + factor * (pos[2 * i + 1] - miny);
    }
}

/* Deformation gradient of element e (:716-719). */
static void or_defgrad(const double *pos, const int *el, const double *inv, int e, double *f11, double *f12,
                       double *f21, double *f22) {
    const int i1 = el[3 * e], i2 = el[3 * e + 1], i3 = el[3 * e + 2];
    const double *M = inv + 6 * (size_t)e;
    *f11 = pos[2 * i1] * M[0] + pos[2 * i2] * M[2] + pos[2 * i3] * M[4];
    *f12 = pos[2 * i1] * M[1] + pos[2 * i2] * M[3] + pos[2 * i3] * M[5];
    *f21 = pos[2 * i1 + 1] * M[0] + pos[2 * i2 + 1] * M[2] + pos[2 * i3 + 1] * M[4];
    *f22 = pos[2 * i1 + 1] * M[1] + pos[2 * i2 + 1] * M[3] + pos[2 * i3 + 1] * M[5];
}

/* :702-751 then :754-780. */
void or_gel_forces(const or_model *m, const double *pos, double *F) {
    const double smod = m->smod, bmod = m->bmod, dil = m->gel_dilation;
    for (int e = 0; e < m->n_elems; ++e) {
        double f11, f12, f21, f22;
        or_defgrad(pos, m->elems, m->inv_mats, e, &f11, &f12, &f21, &f22);
        const double *M = m->inv_mats + 6 * (size_t)e;
        const double A = m->areas[e];
        const double det = f11 * f22 - f12 * f21;
        const double coeff1 = -smod * A / det;
        double coeff2 = bmod * (dil + 1 - det) + smod * (f11 * f11 + f12 * f12 + f21 * f21 + f22 * f22) / (2 * det * det);
        coeff2 *= A;
        const double du11 = f11 * coeff1 + f22 * coeff2;
        const double du12 = f12 * coeff1 - f21 * coeff2;
        const double du21 = f21 * coeff1 - f12 * coeff2;
        const double du22 = f22 * coeff1 + f11 * coeff2;
        for (int r = 0; r < 3; ++r) {
            const int v = m->elems[3 * e + r];
            const double mx = (double)(m->fcodes[v] & 1), my = (double)((m->fcodes[v] & 2) >> 1);
            F[2 * v] = F[2 * v] + du11 * M[2 * r] * mx;
            F[2 * v] = F[2 * v] + du12 * M[2 * r + 1] * mx;
            F[2 * v + 1] = F[2 * v + 1] + du21 * M[2 * r] * my;
            F[2 * v + 1] = F[2 * v + 1] + du22 * M[2 * r + 1] * my;
        }
    }
    for (int p = 0; p < m->n_mpairs; ++p) {
        const int i1 = m->mpairs[2 * p], i2 = m->mpairs[2 * p + 1];
        double t = F[2 * i1];
        F[2 * i1] = F[2 * i1] + F[2 * i2];
        F[2 * i2] = F[2 * i2] + t;
        t = F[2 * i1 + 1];
        F[2 * i1 + 1] = F[2 * i1 + 1] + F[2 * i2 + 1];
        F[2 * i2 + 1] = F[2 * i2 + 1] + t;
    }
}

/* :674-699, summed as |e| (cublasDasum, :1053) with the canonical tree. */
double or_gel_energy(const or_model *m, const double *pos) {
    if (m->n_elems <= 0) return 0.0;
    const double smod = m->smod, bmod = m->bmod, dil = m->gel_dilation;
    double *terms = (double *)malloc(sizeof(double) * (size_t)m->n_elems);
    for (int e = 0; e < m->n_elems; ++e) {
        double f11, f12, f21, f22;
        or_defgrad(pos, m->elems, m->inv_mats, e, &f11, &f12, &f21, &f22);
        const double A = m->areas[e];
        const double det = f11 * f22 - f12 * f21;
        double en = smod * A * ((f11 * f11 + f12 * f12 + f21 * f21 + f22 * f22) / det - 2) / 2;
        en += bmod * A * (det - 1 - dil) * (det - 1 - dil) / 2;
        terms[e] = fabs(en);
    }
    const double s = or_canon_sum(terms, m->n_elems);
    free(terms);
    return s;
}

/* :1256-1274 */
double or_preferred_dilation(double ks, double e_stretch_dilated, double area, double dilation, double bmod) {
    double net_bmod;
    if (ks > 0) {
        net_bmod = e_stretch_dilated;
        net_bmod *= 2 / area / (dilation * dilation);
    } else {
        net_bmod = 0;
    }
    return dilation * (bmod + net_bmod) / bmod;
}

static void or_mesh_record(double *records, int *nrec, int max_records, double curr, double maxc,
                           const or_report *rep, int is_shear) {
    if (*nrec >= max_records) return;
    double *r = records + 9 * (size_t)(*nrec);
    r[0] = curr; r[1] = maxc; r[2] = rep->e_stretch; r[3] = rep->e_bend; r[4] = rep->e_gel;
    r[5] = rep->rms_force; r[6] = rep->max_force; r[7] = rep->steps; r[8] = is_shear;
    (*nrec)++;
}

/* :1276-1376 (strain mode): the first displacement is min_disp, later ones
 * inc; compression lowers the height used by affine_displace as it goes. */
int or_mesh_sweep(const or_model *m, double *pos, double miny, double range, const or_fire_params *p,
                  const double compr[3], const double shear[3], double *records, int max_records,
                  double *shear_pos) {
    const int n = m->n_points;
    double *v = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    double *F = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    const double smult = range;
    int nrec = 0;
    or_report rep;
    double min_disp = compr[0] * smult, max_disp = compr[1] * smult, inc = compr[2] * smult;
    double curr_disp = 0.0;
    if (max_disp > 0) {
        or_affine_displace(n, pos, miny, range, 0, -min_disp);
        range -= min_disp;
        for (curr_disp = min_disp; curr_disp <= max_disp + OR_FLT_TOL; curr_disp += inc) {
            or_fire(m, pos, v, F, p, &rep);
            or_mesh_record(records, &nrec, max_records, 0.0, curr_disp, &rep, 0);
            if (curr_disp < max_disp) {
                or_affine_displace(n, pos, miny, range, 0, -inc);
                range -= inc;
            }
            if (!(inc > 0)) break; /* the reference loops forever when inc == 0 */
        }
    }
    const double max_comp = max_disp > min_disp ? curr_disp - inc : max_disp;
    min_disp = shear[0] * smult;
    max_disp = shear[1] * smult;
    inc = shear[2] * smult;
    if (max_disp > 0) {
        or_affine_displace(n, pos, miny, range, min_disp, 0);
        for (curr_disp = min_disp; curr_disp <= max_disp + OR_FLT_TOL; curr_disp += inc) {
            or_fire(m, pos, v, F, p, &rep);
            if (shear_pos && nrec < max_records)
                memcpy(shear_pos + 2 * (size_t)n * nrec, pos, sizeof(double) * 2 * (size_t)n);
            or_mesh_record(records, &nrec, max_records, curr_disp, max_comp, &rep, 1);
            if (curr_disp < max_disp) or_affine_displace(n, pos, miny, range, inc, 0);
            if (!(inc > 0)) break;
        }
    }
    free(v);
    free(F);
    return nrec;
}
