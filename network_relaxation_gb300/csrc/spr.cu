/*
 * Linear response of a network (src/sparse_relax.cpp, SPR) on sm_103a.
 *
 * The reference builds the harmonic stiffness matrix K of bond stretching
 * (SPR:280-323), linearised bending (:326-386) and background shear
 * (:390-429), projects out the clamped top and bottom rows (:560-605) and,
 * for every (compression, shear) of its protocol, solves the reduced system
 * K_ff u = -(P^T K) bc with SuiteSparseQR (:793), then reports the residual
 * and the linearised energies (:820-870).
 *
 * Here:
 *  - K is assembled on the host in the reference's accumulation order
 *    (a key's contributions added in call order, as its std::map does;
 *    |value| <= 1e-10 dropped), so its entries are bit-identical to the
 *    reference's and the oracle's.
 *  - The reduced system lives on the device in SELL-32 (rows in slices of
 *    32, each slice padded to its longest row, column-major inside the
 *    slice): a warp reads a slice's values and columns coalesced.  Rows are
 *    sorted by length inside windows of 256 (SELL-C-sigma), so slices pad
 *    little.
 *  - bc is linear in (compression, shear), so the protocol needs two
 *    solves: the unit compression and the unit shear loads, solved
 *    together (one matrix read per iteration for both) by a conjugate
 *    gradient with a 2x2 block-Jacobi (per node) preconditioner, in its
 *    single-reduction form (two grid barriers per iteration), in one
 *    persistent cooperative kernel with budgeted grid barriers.  Every protocol point is then a
 *    linear combination, checked by its own residual ||rhs - K_ff u||
 *    (one SpMV) and followed by the energies (canonical tile sums).
 *  - On a rank-deficient system (floppy modes) CG from zero returns the
 *    minimum-norm solution, i.e. the reference's -n option (null-space
 *    removal, SPR:608-671, whose loop at :805 never runs); energies are
 *    unaffected by the null space.
 * Reductions use a fixed order for a given launch shape, so repeated runs
 * give identical bits.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "nr_device.cuh"
#include "nr_internal.h"

namespace nr {
namespace {

constexpr double kSprDrop = 1e-10; /* FLT_TOL, sparse_relax.cpp:45 */
constexpr int kSprThreads = 512;
constexpr int kSlice = 32;
constexpr int kSigma = 256; /* rows sorted by length within windows of this size */

/* ------------------------------------------------------------ assembly */

/* Calls f(row, col, value) (row <= col) in the order of sparse_relax.cpp's
 * update_matrix calls: calc_stretching_elements for every bond, then
 * calc_bending_elements (kb > 0), then calc_shearing_elements (mu > 0).
 * tri_wrap holds two wraps per triple; SPR keeps the first (:257). */
template <class F>
void spr_contributions(const nr_host_network &h, const std::vector<int> &tri_hjk, const std::vector<signed char> &tri_wrap,
                       double ks, double kb, double mu, F &&f) {
    const double *p = h.points.data();
    const double offset = h.offset;
    auto upd = [&](long a, long b, double v) { a < b ? f(a, b, v) : f(b, a, v); };
    for (int e = 0; e < h.n_edges(); ++e) {
        const int a = h.edge_ij[2 * e], b = h.edge_ij[2 * e + 1];
        const double dx = p[2 * b] + offset * h.edge_wrap[e] - p[2 * a];
        const double dy = p[2 * b + 1] - p[2 * a + 1];
        const double l = std::sqrt(dx * dx + dy * dy);
        const double inv_l_cubed = 1 / (l * l * l);
        const long x1 = 2L * a, x2 = 2L * b, y1 = 2L * a + 1, y2 = 2L * b + 1;
        double m = ks * inv_l_cubed * dx * dx;
        upd(x1, x2, -m);
        upd(x1, x1, m);
        upd(x2, x2, m);
        m = ks * inv_l_cubed * dx * dy;
        upd(x1, y2, -m);
        upd(y1, x2, -m);
        upd(x1, y1, m);
        upd(x2, y2, m);
        m = ks * inv_l_cubed * dy * dy;
        upd(y1, y2, -m);
        upd(y1, y1, m);
        upd(y2, y2, m);
    }
    if (kb > 0) {
        const int nt = (int)(tri_hjk.size() / 3);
        for (int t = 0; t < nt; ++t) {
            const long hh = tri_hjk[3 * t], j = tri_hjk[3 * t + 1], k = tri_hjk[3 * t + 2];
            const double dx = p[2 * j] + offset * tri_wrap[2 * t] - p[2 * hh];
            const double dy = p[2 * j + 1] - p[2 * hh + 1];
            const double len_sq = dx * dx + dy * dy;
            const double xx = kb * dx * dx / len_sq;
            const double yy = kb * dy * dy / len_sq;
            const double xy = kb * dx * dy / len_sq;
            upd(2 * hh, 2 * hh, 4 * yy);
            upd(2 * j, 2 * j, yy);
            upd(2 * k, 2 * k, yy);
            upd(2 * hh + 1, 2 * hh + 1, 4 * xx);
            upd(2 * j + 1, 2 * j + 1, xx);
            upd(2 * k + 1, 2 * k + 1, xx);
            upd(2 * hh, 2 * hh + 1, -4 * xy);
            upd(2 * hh, 2 * j, -2 * yy);
            upd(2 * hh, 2 * k, -2 * yy);
            upd(2 * hh, 2 * j + 1, 2 * xy);
            upd(2 * hh, 2 * k + 1, 2 * xy);
            upd(2 * hh + 1, 2 * j, 2 * xy);
            upd(2 * hh + 1, 2 * k, 2 * xy);
            upd(2 * hh + 1, 2 * j + 1, -2 * xx);
            upd(2 * hh + 1, 2 * k + 1, -2 * xx);
            upd(j * 2, j * 2 + 1, -xy);
            upd(j * 2, k * 2, yy);
            upd(j * 2, k * 2 + 1, -xy);
            upd(j * 2 + 1, k * 2, -xy);
            upd(j * 2 + 1, k * 2 + 1, xx);
            upd(k * 2, k * 2 + 1, -xy);
        }
    }
    if (mu > 0) {
        for (int e = 0; e < h.n_edges(); ++e) {
            const long a = h.edge_ij[2 * e], b = h.edge_ij[2 * e + 1];
            const double dx = p[2 * b] + h.edge_wrap[e] * offset - p[2 * a];
            const double dy = p[2 * a + 1] - p[2 * b + 1];
            double inv_len_sq = h.edge_l0[e];
            inv_len_sq = 1 / inv_len_sq / inv_len_sq;
            const double rh_x_sq = dx * dx * inv_len_sq;
            const double rh_y_sq = dy * dy * inv_len_sq;
            double m = mu * (1 - rh_x_sq);
            upd(a * 2, a * 2, m);
            upd(b * 2, b * 2, m);
            upd(a * 2, b * 2, -m);
            m = mu * (1 - rh_y_sq);
            upd(a * 2 + 1, a * 2 + 1, m);
            upd(b * 2 + 1, b * 2 + 1, m);
            upd(a * 2 + 1, b * 2 + 1, -m);
        }
    }
}

/* Upper triangle of K by rows: row r holds (col, value), col >= r,
 * ascending. */
struct UpperK {
    long n_dof = 0;
    std::vector<long> ptr;
    std::vector<long> col;
    std::vector<double> val;
};

/* get_sparse_stiffness_mat (SPR:434-480).  Contributions are bucketed by
 * row keeping their call order (a counting sort), then within a row
 * ordered by column stably and summed in call order: the value the
 * reference's std::map holds for each key. */
void assemble_upper(const nr_host_network &h, double ks, double kb, double mu, UpperK &K) {
    std::vector<int> tri_hjk;
    std::vector<signed char> tri_wrap;
    if (kb > 0) { /* get_sparse_stiffness_mat recomputes the triples (:444-446) */
        nr_host_network copy;
        copy.n_points = h.n_points;
        copy.offset = h.offset;
        copy.points = h.points;
        copy.edge_ij = h.edge_ij;
        copy.edge_l0 = h.edge_l0;
        copy.edge_wrap = h.edge_wrap;
        nr_get_triples(&copy);
        tri_hjk.swap(copy.tri_hjk);
        tri_wrap.swap(copy.tri_wrap);
    }
    const long n_dof = 2L * h.n_points;
    K.n_dof = n_dof;
    std::vector<long> cnt(n_dof + 1, 0);
    spr_contributions(h, tri_hjk, tri_wrap, ks, kb, mu, [&](long r, long, double) { cnt[r + 1]++; });
    for (long r = 0; r < n_dof; ++r) cnt[r + 1] += cnt[r];
    std::vector<long> fill(cnt.begin(), cnt.end() - 1);
    std::vector<long> c_col(cnt[n_dof]);
    std::vector<double> c_val(cnt[n_dof]);
    spr_contributions(h, tri_hjk, tri_wrap, ks, kb, mu, [&](long r, long c, double v) {
        const long at = fill[r]++;
        c_col[at] = c;
        c_val[at] = v;
    });
    K.ptr.assign(n_dof + 1, 0);
    K.col.clear();
    K.val.clear();
    std::vector<long> idx;
    for (long r = 0; r < n_dof; ++r) {
        const long b = cnt[r], e = cnt[r + 1];
        idx.resize(e - b);
        for (long q = b; q < e; ++q) idx[q - b] = q;
        std::stable_sort(idx.begin(), idx.end(), [&](long x, long y) { return c_col[x] < c_col[y]; });
        for (size_t q = 0; q < idx.size();) {
            double v = c_val[idx[q]];
            size_t s = q + 1;
            while (s < idx.size() && c_col[idx[s]] == c_col[idx[q]]) v += c_val[idx[s++]];
            if (std::fabs(v) > kSprDrop) {
                K.col.push_back(c_col[idx[q]]);
                K.val.push_back(v);
            }
            q = s;
        }
        K.ptr[r + 1] = (long)K.col.size();
    }
}

/* ------------------------------------------------------------- device */

struct SprScal {
    double rho[2], mu[2], alpha[2], beta[2], rr[2], bb[2];
    int active[2], iters[2];
    int done, pad;
};

/* Reduced system in device order: free node k owns rows 2k (x) and 2k + 1
 * (y); vectors hold the two right-hand sides (double2 per row). */
struct SprDev {
    int nr, n_slices;
    const long *slice_ptr;
    const int *slice_w;
    const int *col;
    const double *val;
    const double2 *mdiag; /* per node: inverse 2x2 diagonal block, (a00, a11) */
    const double *moff;   /* per node: its off-diagonal a01 */
    const double2 *b;
    double2 *x, *r, *z, *p, *q, *s;
    double *part; /* kParts per block */
    SprScal *sc;
    FireState *bar; /* barrier words */
};

constexpr int kParts = 8;

__device__ __forceinline__ double2 spmv_row(const SprDev &d, int s, int lane, const double2 *v) {
    const long base = d.slice_ptr[s];
    const int w = d.slice_w[s];
    double a0 = 0.0, a1 = 0.0;
    for (int k = 0; k < w; ++k) {
        const long at = base + (long)k * kSlice + lane;
        const double m = d.val[at];
        const double2 pv = v[d.col[at]];
        a0 = fma(m, pv.x, a0);
        a1 = fma(m, pv.y, a1);
    }
    return make_double2(a0, a1);
}

/* Block sums of kParts values into part[blockIdx * kParts + k]. */
__device__ void block_parts(double *s_red, double *part, const double *v) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < kParts; ++k) {
        const double t = warp_sum(v[k]);
        if (lane == 0) s_red[warp * kParts + k] = t;
    }
    __syncthreads();
    if (threadIdx.x < kParts) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t = t + s_red[w * kParts + threadIdx.x];
        part[blockIdx.x * kParts + threadIdx.x] = t;
    }
    __syncthreads();
}

/* Totals of the kParts partial columns over G blocks (warp k sums column
 * k: lanes stride the blocks, then a butterfly); every thread gets them.
 * Needs kParts warps. */
__device__ void total_parts(double *s_red, const double *part, int G, double *t) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp < kParts) {
        double v = 0.0;
        for (int b = lane; b < G; b += 32) v = v + __ldcg(part + b * kParts + warp);
        v = warp_sum(v);
        if (lane == 0) s_red[warp] = v;
    }
    __syncthreads();
    for (int k = 0; k < kParts; ++k) t[k] = s_red[k];
    __syncthreads();
}

/* z = M^-1 r for node k's two rows (2x2 block Jacobi), both right-hand sides. */
__device__ __forceinline__ void precond(const SprDev &d, int k, double2 rx, double2 ry, double2 &zx, double2 &zy) {
    const double2 m = d.mdiag[k];
    const double o = d.moff[k];
    zx = make_double2(fma(m.x, rx.x, o * ry.x), fma(m.x, rx.y, o * ry.y));
    zy = make_double2(fma(o, rx.x, m.y * ry.x), fma(o, rx.y, m.y * ry.y));
}

/* s = K z over the rows, with the row terms of rho = r.z and mu = z.s. */
__device__ __forceinline__ void spmv_phase(const SprDev &d, int gwarp, int nwarps, int lane, double *acc) {
    for (int sl = gwarp; sl < d.n_slices; sl += nwarps) {
        const double2 sv = spmv_row(d, sl, lane, d.z);
        const int row = sl * kSlice + lane;
        if (row < d.nr) {
            d.s[row] = sv;
            const double2 rv = d.r[row], zv = d.z[row];
            acc[0] = fma(rv.x, zv.x, acc[0]);
            acc[1] = fma(rv.y, zv.y, acc[1]);
            acc[2] = fma(zv.x, sv.x, acc[2]);
            acc[3] = fma(zv.y, sv.y, acc[3]);
        }
    }
}

/* Block-Jacobi-preconditioned conjugate gradient in the single-reduction
 * form of Chronopoulos and Gear (J. Comput. Appl. Math. 25, 1989): per
 * iteration one fused vector pass (p = z + beta p, q = s + beta q,
 * x += alpha p, r -= alpha q, z = M^-1 r) and one SpMV s = K z that also
 * yields r.z and z.s, so two grid barriers.  Two right-hand sides at once;
 * each stops at ||r|| <= tol ||b|| (then alpha = beta = 0 freeze it). */
__global__ void __launch_bounds__(kSprThreads) k_spr_pcg(SprDev d, double tol, int max_iter,
                                                         unsigned long long budget_ns) {
    __shared__ double s_red[(kSprThreads / 32) * kParts];
    const unsigned G = gridDim.x;
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = G * blockDim.x;
    const int lane = threadIdx.x & 31;
    const int gwarp = tid >> 5, nwarps = nth >> 5;
    const int nn = d.nr / 2;
    bool last;
    volatile SprScal *vs = d.sc;
    const double2 zero = make_double2(0.0, 0.0);
    double acc[kParts];
    /* r = b, z = M^-1 r, x = p = q = 0; b.b */
    for (int k = 0; k < kParts; ++k) acc[k] = 0.0;
    for (int k = tid; k < nn; k += nth) {
        const double2 bx = d.b[2 * k], by = d.b[2 * k + 1];
        double2 zx, zy;
        precond(d, k, bx, by, zx, zy);
        d.r[2 * k] = bx;
        d.r[2 * k + 1] = by;
        d.z[2 * k] = zx;
        d.z[2 * k + 1] = zy;
        d.x[2 * k] = d.x[2 * k + 1] = zero;
        d.p[2 * k] = d.p[2 * k + 1] = zero;
        d.q[2 * k] = d.q[2 * k + 1] = zero;
        acc[4] = fma(bx.x, bx.x, fma(by.x, by.x, acc[4]));
        acc[5] = fma(bx.y, bx.y, fma(by.y, by.y, acc[5]));
    }
    if (!barrier_arrive(d.bar, G, budget_ns, last, 21)) return;
    if (last) barrier_release(d.bar);
    spmv_phase(d, gwarp, nwarps, lane, acc);
    block_parts(s_red, d.part, acc);
    if (!barrier_arrive(d.bar, G, budget_ns, last, 22)) return;
    if (last) {
        double t[kParts];
        total_parts(s_red, d.part, G, t);
        if (threadIdx.x == 0) {
            SprScal *sc = d.sc;
            for (int k = 0; k < 2; ++k) {
                sc->rho[k] = t[k];
                sc->mu[k] = t[2 + k];
                sc->bb[k] = t[4 + k];
                sc->rr[k] = t[4 + k];
                sc->iters[k] = 0;
                sc->beta[k] = 0.0;
                sc->active[k] = t[4 + k] > 0 && t[k] != 0 && t[2 + k] != 0;
                sc->alpha[k] = sc->active[k] ? t[k] / t[2 + k] : 0.0;
            }
            sc->done = !(sc->active[0] || sc->active[1]) || max_iter <= 0;
        }
        barrier_release(d.bar);
    }
    for (;;) {
        if (vs->done) break;
        const double al0 = vs->alpha[0], al1 = vs->alpha[1], be0 = vs->beta[0], be1 = vs->beta[1];
        for (int k = 0; k < kParts; ++k) acc[k] = 0.0;
        for (int k = tid; k < nn; k += nth) {
            double2 rr2[2], zz2[2];
            for (int c = 0; c < 2; ++c) {
                const int i = 2 * k + c;
                const double2 zv = d.z[i], sv = d.s[i];
                double2 pv = d.p[i], qv = d.q[i], xv = d.x[i], rv = d.r[i];
                pv.x = fma(be0, pv.x, zv.x);
                pv.y = fma(be1, pv.y, zv.y);
                qv.x = fma(be0, qv.x, sv.x);
                qv.y = fma(be1, qv.y, sv.y);
                xv.x = fma(al0, pv.x, xv.x);
                xv.y = fma(al1, pv.y, xv.y);
                rv.x = fma(-al0, qv.x, rv.x);
                rv.y = fma(-al1, qv.y, rv.y);
                d.p[i] = pv;
                d.q[i] = qv;
                d.x[i] = xv;
                d.r[i] = rv;
                rr2[c] = rv;
                acc[4] = fma(rv.x, rv.x, acc[4]);
                acc[5] = fma(rv.y, rv.y, acc[5]);
            }
            precond(d, k, rr2[0], rr2[1], zz2[0], zz2[1]);
            d.z[2 * k] = zz2[0];
            d.z[2 * k + 1] = zz2[1];
        }
        if (!barrier_arrive(d.bar, G, budget_ns, last, 23)) return;
        if (last) barrier_release(d.bar);
        spmv_phase(d, gwarp, nwarps, lane, acc);
        block_parts(s_red, d.part, acc);
        if (!barrier_arrive(d.bar, G, budget_ns, last, 24)) return;
        if (last) {
            double t[kParts];
            total_parts(s_red, d.part, G, t);
            if (threadIdx.x == 0) {
                SprScal *sc = d.sc;
                for (int k = 0; k < 2; ++k) {
                    if (!sc->active[k]) {
                        sc->alpha[k] = sc->beta[k] = 0.0;
                        continue;
                    }
                    sc->iters[k]++;
                    sc->rr[k] = t[4 + k];
                    const double rho = t[k], mu = t[2 + k];
                    const double beta = rho / sc->rho[k];
                    const double den = mu - beta * rho / sc->alpha[k];
                    if (!(t[4 + k] > tol * tol * sc->bb[k]) || rho == 0 || !(den != 0) || !isfinite(den)) {
                        sc->active[k] = 0;
                        sc->alpha[k] = sc->beta[k] = 0.0;
                        continue;
                    }
                    sc->beta[k] = beta;
                    sc->alpha[k] = rho / den;
                    sc->rho[k] = rho;
                }
                sc->done = !(sc->active[0] || sc->active[1]) || sc->iters[0] >= max_iter || sc->iters[1] >= max_iter;
            }
            barrier_release(d.bar);
        }
    }
}

/* ---------------------------------------------- per protocol point */

struct SprPointDev {
    int n, nr;
    double miny, maxy, compression, shear;
    int affine;
    const double2 *pos;
    const int *dof_map;        /* 2N: reduced index or -1 */
    const unsigned char *top; /* N */
    const double2 *xsol;      /* nr: (unit compression, unit shear) solutions */
    double *u_red;            /* nr */
    double2 *u_final;         /* N */
};

/* u = c X_c + s X_s on the free dofs; u_final = bc + P u (SPR:812-813),
 * bc from affine_displacement (:528-538) or add_displacement (:513-525). */
__global__ void k_spr_field(SprPointDev a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const double2 pt = a.pos[i];
    double2 bc = make_double2(0.0, 0.0);
    if (a.affine) {
        const double c_strain = a.compression / (a.maxy - a.miny), s_strain = a.shear / (a.maxy - a.miny);
        bc.x = s_strain * (pt.y - a.miny);
        bc.y = c_strain * (a.miny - pt.y);
    } else if (a.top[i]) {
        bc.x = 1 * a.shear;
        bc.y = -1 * a.compression;
    }
    double2 uf = bc;
    const int rx = a.dof_map[2 * i], ry = a.dof_map[2 * i + 1];
    if (rx >= 0) {
        const double2 s = a.xsol[rx];
        const double u = a.compression * s.x + a.shear * s.y;
        a.u_red[rx] = u;
        uf.x = uf.x + u;
    }
    if (ry >= 0) {
        const double2 s = a.xsol[ry];
        const double u = a.compression * s.x + a.shear * s.y;
        a.u_red[ry] = u;
        uf.y = uf.y + u;
    }
    a.u_final[i] = uf;
}

/* Residual rhs - K_ff u of one point (rhs = c b_c + s b_s): per-block sums
 * of its squares. */
__global__ void __launch_bounds__(kSprThreads) k_spr_residual(SprDev d, const double *u, double c, double s,
                                                              double *part) {
    __shared__ double s_red[(kSprThreads / 32) * kParts];
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, gwarp = tid >> 5, nwarps = nth >> 5;
    double acc = 0.0;
    for (int sl = gwarp; sl < d.n_slices; sl += nwarps) {
        const long base = d.slice_ptr[sl];
        const int w = d.slice_w[sl];
        double ku = 0.0;
        for (int k = 0; k < w; ++k) {
            const long at = base + (long)k * kSlice + lane;
            ku = fma(d.val[at], u[d.col[at]], ku);
        }
        const int row = sl * kSlice + lane;
        if (row < d.nr) {
            const double2 b = d.b[row];
            const double rv = (c * b.x + s * b.y) - ku;
            acc = fma(rv, rv, acc);
        }
    }
    double v[kParts] = {acc, 0, 0, 0, 0, 0, 0, 0};
    block_parts(s_red, part, v);
}

__global__ void k_spr_sum_parts(const double *part, int G, double *out) {
    __shared__ double s_red[kParts];
    double t[kParts];
    total_parts(s_red, part, G, t);
    if (threadIdx.x == 0) *out = t[0];
}

struct SprEnergyDev {
    int n_edges, n_triples;
    double offset, ks, kb, mu;
    const double2 *pos;
    const int4 *bond; /* {i, j, wrap, 0} */
    const double *l0;
    const int4 *tri;  /* {h, j, k, wrap_j} */
    const double2 *u;
};

/* get_stretch_shear_energy (SPR:49-71) per bond. */
__device__ __forceinline__ double ss_term(const SprEnergyDev &a, int e) {
    const int4 b = a.bond[e];
    const double2 p1 = a.pos[b.x], p2 = a.pos[b.y], u1 = a.u[b.x], u2 = a.u[b.y];
    const double dx = p2.x + b.z * a.offset - p1.x;
    const double dy = p2.y - p1.y;
    const double dux = u2.x - u1.x, duy = u2.y - u1.y;
    const double de = (dux * dx + duy * dy) / a.l0[e];
    return .5 * a.ks * de * de + .5 * a.mu * (dux * dux + duy * duy - de * de);
}
/* get_bending_energy (SPR:74-96) per triple. */
__device__ __forceinline__ double bend_term(const SprEnergyDev &a, int t) {
    const int4 r = a.tri[t];
    const double2 ph = a.pos[r.x], pj = a.pos[r.y];
    const double2 uh = a.u[r.x], uj = a.u[r.y], uk = a.u[r.z];
    const double dx = pj.x + a.offset * r.w - ph.x;
    const double dy = pj.y - ph.y;
    const double length_sq = dx * dx + dy * dy;
    const double dux = uj.x + uk.x - 2 * uh.x, duy = uj.y + uk.y - 2 * uh.y;
    const double c = dux * dy - duy * dx;
    return .5 * a.kb * c * c / length_sq;
}

/* Canonical tile partials: tiles of bonds then tiles of triples. */
__global__ void __launch_bounds__(kTile) k_spr_energy_tiles(SprEnergyDev a, int use_ss, int use_bend, double *epart,
                                                            int stride) {
    __shared__ double s_red[kTile / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tb = use_ss ? (a.n_edges + kTile - 1) / kTile : 0;
    const int tt = use_bend ? (a.n_triples + kTile - 1) / kTile : 0;
    for (int t = blockIdx.x; t < tb + tt; t += gridDim.x) {
        const bool is_bond = t < tb;
        const int tile = is_bond ? t : t - tb;
        const int item = tile * kTile + threadIdx.x;
        double e = 0.0;
        if (is_bond) {
            if (item < a.n_edges) e = ss_term(a, item);
        } else if (item < a.n_triples) {
            e = bend_term(a, item);
        }
        e = warp_sum(e);
        if (lane == 0) s_red[warp] = e;
        __syncthreads();
        if (threadIdx.x == 0) epart[(is_bond ? 0 : stride) + tile] = tree8(s_red);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kTile) k_spr_energy_final(const double *epart, int tb, int tt, int stride,
                                                            double *out) {
    __shared__ double s_red[kTile / 32];
    const double es = tb > 0 ? final_sum(epart, tb, 8, s_red) : 0.0;
    const double eb = tt > 0 ? final_sum(epart + stride, tt, 8, s_red) : 0.0;
    if (threadIdx.x == 0) {
        out[0] = es;
        out[1] = eb;
    }
}

int sm_count_spr() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

}  // namespace
}  // namespace nr

using namespace nr;

#define SPR_TRY(call)                                                                         \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(NR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));     \
    } while (0)

struct nr_spr {
    int n = 0, nr = 0, n_slices = 0;
    long nnz_upper = 0, sell_len = 0;
    double ks = 0, kb = 0, mu = 0, offset = 0, miny = 0, maxy = 0, minx = 0, maxx = 0;
    int n_edges = 0, n_triples = 0;
    UpperK K;
    std::vector<int> dof_map;           /* 2N: reduced row (host order) or -1 */
    std::vector<int> perm;              /* device position -> reduced row */
    std::vector<unsigned char> top;     /* N */
    std::vector<double> points;         /* 2N, for the unit loads of either mode */
    int solved_affine = -1;             /* mode of the unit solutions on the device, -1: none */
    int iterations[2] = {0, 0};
    double rel_residual[2] = {0, 0};
    char *arena = nullptr;
    SprDev dev{};
    SprEnergyDev edev{};
    int *d_dof_map = nullptr;
    unsigned char *d_top = nullptr;
    double *d_u_red = nullptr, *d_rpart = nullptr, *d_scalar = nullptr, *d_epart = nullptr;
    double2 *d_u_final = nullptr;
    int e_stride = 1;
    int rpart_blocks = 1; /* capacity of d_rpart in blocks */
    int pcg_blocks = 1;   /* grid of k_spr_pcg (capacity of dev.part) */
    ~nr_spr() {
        if (arena) cudaFree(arena);
    }
};

namespace {

/* Unit loads (compression 1, shear 0) and (0, 1): rhs = -(P^T K) bc
 * (SPR:791), the row sums of the free rows in column order. */
void unit_rhs(nr_spr &S, int affine, std::vector<double> &rhs2) {
    const int n = S.n;
    std::vector<double> bc_c(2 * (size_t)n, 0.0), bc_s(2 * (size_t)n, 0.0);
    for (int i = 0; i < n; ++i) {
        const double y = S.points[2 * i + 1];
        if (affine) {
            bc_s[2 * i] = (1.0 / (S.maxy - S.miny)) * (y - S.miny);
            bc_c[2 * i + 1] = (1.0 / (S.maxy - S.miny)) * (S.miny - y);
        } else if (S.top[i]) {
            bc_s[2 * i] = 1.0;
            bc_c[2 * i + 1] = -1.0;
        }
    }
    /* full rows of the free dofs: upper row entries plus transposed ones */
    rhs2.assign(2 * (size_t)S.nr, 0.0);
    const UpperK &K = S.K;
    std::vector<double> acc_c(S.nr, 0.0), acc_s(S.nr, 0.0);
    for (long r = 0; r < K.n_dof; ++r)
        for (long q = K.ptr[r]; q < K.ptr[r + 1]; ++q) {
            const long c = K.col[q];
            const double v = K.val[q];
            const int rr = S.dof_map[r], rc = S.dof_map[c];
            if (rr >= 0) {
                acc_c[rr] += v * bc_c[c];
                acc_s[rr] += v * bc_s[c];
            }
            if (c != r && rc >= 0) {
                acc_c[rc] += v * bc_c[r];
                acc_s[rc] += v * bc_s[r];
            }
        }
    for (int r = 0; r < S.nr; ++r) {
        rhs2[2 * (size_t)r] = -acc_c[r];
        rhs2[2 * (size_t)r + 1] = -acc_s[r];
    }
}

struct Img {
    std::vector<char> bytes;
    size_t add(size_t nb) {
        const size_t off = (bytes.size() + 255) / 256 * 256;
        bytes.resize(off + nb);
        return off;
    }
    template <class T>
    size_t put(const T *src, size_t cnt) {
        const size_t off = add(cnt * sizeof(T));
        if (cnt) memcpy(bytes.data() + off, src, cnt * sizeof(T));
        return off;
    }
};

int spr_blocks(int *blocks) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spr_pcg, kSprThreads, 0);
    if (e != cudaSuccess) return fail(NR_ERR_CUDA, std::string("occupancy: ") + cudaGetErrorString(e));
    *blocks = std::max(1, per_sm * sm_count_spr());
    return NR_OK;
}

}  // namespace

extern "C" {

long nr_spr_assemble(const nr_host_network *net, double ks, double kb, double mu, long *rows, long *cols,
                     double *vals) {
    if (!net || net->n_points <= 0) return fail(NR_ERR_INVALID, "nr_spr_assemble: bad network");
    UpperK K;
    assemble_upper(*net, ks, kb, mu, K);
    if (rows && cols && vals)
        for (long r = 0; r < K.n_dof; ++r)
            for (long q = K.ptr[r]; q < K.ptr[r + 1]; ++q) {
                rows[q] = r;
                cols[q] = K.col[q];
                vals[q] = K.val[q];
            }
    return (long)K.col.size();
}

int nr_spr_create(const nr_host_network *net, double ks, double kb, double mu, void *stream, nr_spr **out) {
    if (!net || !out || net->n_points <= 0 || !(ks >= 0) || !(kb >= 0) || !(mu >= 0))
        return fail(NR_ERR_INVALID, "nr_spr_create: bad arguments");
    *out = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    auto *S = new nr_spr();
    const nr_host_network &h = *net;
    S->n = h.n_points;
    S->ks = ks;
    S->kb = kb;
    S->mu = mu;
    S->offset = h.offset;
    /* read_network's ranges (SPR:121-124, :142-145) */
    S->minx = FLT_MAX;
    S->maxx = FLT_MIN;
    S->miny = FLT_MAX;
    S->maxy = FLT_MIN;
    for (int i = 0; i < S->n; ++i) {
        const double x = h.points[2 * i], y = h.points[2 * i + 1];
        if (x < S->minx) S->minx = x;
        if (x > S->maxx) S->maxx = x;
        if (y < S->miny) S->miny = y;
        if (y > S->maxy) S->maxy = y;
    }
    assemble_upper(h, ks, kb, mu, S->K);
    S->nnz_upper = (long)S->K.col.size();
    /* free nodes: neither bottom nor top (SPR:721-724) */
    S->dof_map.assign(2 * (size_t)S->n, -1);
    S->top.assign(S->n, 0);
    for (int i = 0; i < S->n; ++i) {
        const double y = h.points[2 * i + 1];
        const bool bottom = y < S->miny + 1e-10, top = y > S->maxy - 1e-10;
        S->top[i] = top;
        if (!bottom && !top) {
            S->dof_map[2 * i] = S->nr++;
            S->dof_map[2 * i + 1] = S->nr++;
        }
    }
    /* reduced full-symmetric rows, columns ascending */
    std::vector<long> rcnt(S->nr + 1, 0);
    const UpperK &K = S->K;
    for (long r = 0; r < K.n_dof; ++r)
        for (long q = K.ptr[r]; q < K.ptr[r + 1]; ++q) {
            const long c = K.col[q];
            const int rr = S->dof_map[r], rc = S->dof_map[c];
            if (rr >= 0 && rc >= 0) {
                rcnt[rr + 1]++;
                if (c != r) rcnt[rc + 1]++;
            }
        }
    for (int r = 0; r < S->nr; ++r) rcnt[r + 1] += rcnt[r];
    std::vector<int> rcol(rcnt[S->nr]);
    std::vector<double> rval(rcnt[S->nr]);
    std::vector<double> diag(S->nr, 0.0);
    {
        std::vector<long> fill(rcnt.begin(), rcnt.end() - 1);
        for (long r = 0; r < K.n_dof; ++r)
            for (long q = K.ptr[r]; q < K.ptr[r + 1]; ++q) {
                const long c = K.col[q];
                const int rr = S->dof_map[r], rc = S->dof_map[c];
                if (rr < 0 || rc < 0) continue;
                rcol[fill[rr]] = rc;
                rval[fill[rr]++] = K.val[q];
                if (c != r) {
                    rcol[fill[rc]] = rr;
                    rval[fill[rc]++] = K.val[q];
                } else {
                    diag[rr] = K.val[q];
                }
            }
        std::vector<std::pair<int, double>> tmp;
        for (int r = 0; r < S->nr; ++r) {
            tmp.clear();
            for (long q = rcnt[r]; q < rcnt[r + 1]; ++q) tmp.push_back({rcol[q], rval[q]});
            std::sort(tmp.begin(), tmp.end(), [](const std::pair<int, double> &a, const std::pair<int, double> &b) {
                return a.first < b.first;
            });
            for (size_t k = 0; k < tmp.size(); ++k) {
                rcol[rcnt[r] + k] = tmp[k].first;
                rval[rcnt[r] + k] = tmp[k].second;
            }
        }
    }
    /* SELL-32 with nodes sorted by row length inside windows of kSigma rows
     * (SELL-C-sigma): slices of rows of similar length pad little, the
     * window keeps neighbouring nodes together for the gathers, and a
     * node's x and y rows stay adjacent (rows 2k, 2k + 1 of device node k)
     * for the 2x2 block preconditioner.  perm: device row -> reduced row;
     * columns are renumbered; each row keeps its column order, so its sum
     * is unchanged. */
    const int nn = S->nr / 2;
    const auto row_len = [&](int r) { return rcnt[r + 1] - rcnt[r]; };
    std::vector<int> pnode(nn);
    for (int j = 0; j < nn; ++j) pnode[j] = j;
    const int wnodes = kSigma / 2;
    for (int w0 = 0; w0 < nn; w0 += wnodes) {
        const int w1 = std::min(nn, w0 + wnodes);
        std::stable_sort(pnode.begin() + w0, pnode.begin() + w1, [&](int a, int b) {
            return std::max(row_len(2 * a), row_len(2 * a + 1)) > std::max(row_len(2 * b), row_len(2 * b + 1));
        });
    }
    std::vector<int> perm(S->nr), inv(S->nr);
    for (int k = 0; k < nn; ++k) {
        perm[2 * k] = 2 * pnode[k];
        perm[2 * k + 1] = 2 * pnode[k] + 1;
    }
    for (int k = 0; k < S->nr; ++k) inv[perm[k]] = k;
    S->perm = perm;
    S->n_slices = (S->nr + kSlice - 1) / kSlice;
    std::vector<long> slice_ptr(S->n_slices + 1, 0);
    std::vector<int> slice_w(S->n_slices, 0);
    for (int sl = 0; sl < S->n_slices; ++sl) {
        int w = 0;
        for (int l = 0; l < kSlice; ++l) {
            const int k = sl * kSlice + l;
            if (k < S->nr) w = std::max(w, (int)row_len(perm[k]));
        }
        slice_w[sl] = w;
        slice_ptr[sl + 1] = slice_ptr[sl] + (long)w * kSlice;
    }
    S->sell_len = slice_ptr[S->n_slices];
    std::vector<int> scol(S->sell_len, 0);
    std::vector<double> sval(S->sell_len, 0.0);
    for (int sl = 0; sl < S->n_slices; ++sl)
        for (int l = 0; l < kSlice; ++l) {
            const int k = sl * kSlice + l;
            const int r = k < S->nr ? perm[k] : -1;
            for (int q = 0; q < slice_w[sl]; ++q) {
                const long at = slice_ptr[sl] + (long)q * kSlice + l;
                if (r >= 0 && q < row_len(r)) {
                    scol[at] = inv[rcol[rcnt[r] + q]];
                    sval[at] = rval[rcnt[r] + q];
                } else {
                    scol[at] = k < S->nr ? k : 0; /* padding: a valid index, value 0 */
                }
            }
        }
    /* inverse of each node's 2x2 diagonal block (scalar Jacobi when the
     * block is singular or nearly so) */
    std::vector<double2> mdiag(std::max(1, nn));
    std::vector<double> moff(std::max(1, nn));
    for (int k = 0; k < nn; ++k) {
        const int rx = perm[2 * k];
        const double kxx = diag[rx], kyy = diag[rx + 1];
        double kxy = 0.0;
        for (long q = rcnt[rx]; q < rcnt[rx + 1]; ++q)
            if (rcol[q] == rx + 1) kxy = rval[q];
        const double det = kxx * kyy - kxy * kxy;
        if (kxx > 0 && kyy > 0 && det > 1e-12 * kxx * kyy) {
            mdiag[k] = make_double2(kyy / det, kxx / det);
            moff[k] = -kxy / det;
        } else {
            mdiag[k] = make_double2(kxx > 0 ? 1.0 / kxx : 0.0, kyy > 0 ? 1.0 / kyy : 0.0);
            moff[k] = 0.0;
        }
    }
    std::vector<int> dof_dev(S->dof_map.size());
    for (size_t f = 0; f < dof_dev.size(); ++f) dof_dev[f] = S->dof_map[f] >= 0 ? inv[S->dof_map[f]] : -1;
    /* energies: bonds, SPR's triples (recomputed like the reference) */
    std::vector<int4> bond(h.n_edges());
    for (int e = 0; e < h.n_edges(); ++e)
        bond[e] = make_int4(h.edge_ij[2 * e], h.edge_ij[2 * e + 1], h.edge_wrap[e], 0);
    std::vector<int4> tri;
    if (kb > 0) {
        nr_host_network copy;
        copy.n_points = h.n_points;
        copy.offset = h.offset;
        copy.points = h.points;
        copy.edge_ij = h.edge_ij;
        copy.edge_l0 = h.edge_l0;
        copy.edge_wrap = h.edge_wrap;
        nr_get_triples(&copy);
        for (int t = 0; t < copy.n_triples(); ++t)
            tri.push_back(make_int4(copy.tri_hjk[3 * t], copy.tri_hjk[3 * t + 1], copy.tri_hjk[3 * t + 2],
                                    copy.tri_wrap[2 * t]));
    }
    S->n_edges = h.n_edges();
    S->n_triples = (int)tri.size();
    int blocks = 0;
    int rc = spr_blocks(&blocks);
    if (rc != NR_OK) {
        delete S;
        return rc;
    }
    const int tb = (S->n_edges + kTile - 1) / kTile, tt = (S->n_triples + kTile - 1) / kTile;
    S->e_stride = std::max(1, std::max(tb, tt));
    Img img;
    const size_t o_sp = img.put(slice_ptr.data(), slice_ptr.size());
    const size_t o_sw = img.put(slice_w.data(), slice_w.size());
    const size_t o_col = img.put(scol.data(), scol.size());
    const size_t o_val = img.put(sval.data(), sval.size());
    const size_t o_md = img.put(mdiag.data(), mdiag.size());
    const size_t o_mo = img.put(moff.data(), moff.size());
    const size_t o_b = img.add(sizeof(double2) * (S->nr + 1));
    const size_t o_x = img.add(sizeof(double2) * (S->nr + 1));
    const size_t o_r = img.add(sizeof(double2) * (S->nr + 1));
    const size_t o_p = img.add(sizeof(double2) * (S->nr + 1));
    const size_t o_q = img.add(sizeof(double2) * (S->nr + 1));
    const size_t o_z = img.add(sizeof(double2) * (S->nr + 1));
    const size_t o_s = img.add(sizeof(double2) * (S->nr + 1));
    const size_t o_part = img.add(sizeof(double) * kParts * (size_t)blocks);
    S->pcg_blocks = blocks;
    S->rpart_blocks = 4 * sm_count_spr(); /* k_spr_residual's largest grid */
    const size_t o_rpart = img.add(sizeof(double) * kParts * (size_t)S->rpart_blocks);
    const size_t o_sc = img.add(sizeof(SprScal));
    const size_t o_bar = img.add(sizeof(FireState));
    const size_t o_map = img.put(dof_dev.data(), dof_dev.size());
    const size_t o_top = img.put(S->top.data(), S->top.size());
    const size_t o_ured = img.add(sizeof(double) * (S->nr + 1));
    const size_t o_uf = img.add(sizeof(double2) * (size_t)S->n);
    const size_t o_pos = img.put((const double2 *)h.points.data(), (size_t)S->n);
    const size_t o_bond = img.put(bond.data(), bond.size());
    const size_t o_l0 = img.put(h.edge_l0.data(), h.edge_l0.size());
    const size_t o_tri = img.put(tri.data(), tri.size());
    const size_t o_ep = img.add(sizeof(double) * 2 * (size_t)S->e_stride);
    const size_t o_scalar = img.add(sizeof(double) * 4);
    cudaError_t e = cudaMalloc((void **)&S->arena, img.bytes.size());
    if (e != cudaSuccess) {
        S->arena = nullptr;
        delete S;
        return fail(e == cudaErrorMemoryAllocation ? NR_ERR_OOM : NR_ERR_CUDA,
                    std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    char *base = S->arena;
    SprDev &d = S->dev;
    d.nr = S->nr;
    d.n_slices = S->n_slices;
    d.slice_ptr = (const long *)(base + o_sp);
    d.slice_w = (const int *)(base + o_sw);
    d.col = (const int *)(base + o_col);
    d.val = (const double *)(base + o_val);
    d.mdiag = (const double2 *)(base + o_md);
    d.moff = (const double *)(base + o_mo);
    d.b = (const double2 *)(base + o_b);
    d.x = (double2 *)(base + o_x);
    d.r = (double2 *)(base + o_r);
    d.p = (double2 *)(base + o_p);
    d.q = (double2 *)(base + o_q);
    d.z = (double2 *)(base + o_z);
    d.s = (double2 *)(base + o_s);
    d.part = (double *)(base + o_part);
    d.sc = (SprScal *)(base + o_sc);
    d.bar = (FireState *)(base + o_bar);
    S->d_rpart = (double *)(base + o_rpart);
    S->d_dof_map = (int *)(base + o_map);
    S->d_top = (unsigned char *)(base + o_top);
    S->d_u_red = (double *)(base + o_ured);
    S->d_u_final = (double2 *)(base + o_uf);
    S->d_epart = (double *)(base + o_ep);
    S->d_scalar = (double *)(base + o_scalar);
    SprEnergyDev &ed = S->edev;
    ed.n_edges = S->n_edges;
    ed.n_triples = S->n_triples;
    ed.offset = h.offset;
    ed.ks = ks;
    ed.kb = kb;
    ed.mu = mu;
    ed.pos = (const double2 *)(base + o_pos);
    ed.bond = (const int4 *)(base + o_bond);
    ed.l0 = (const double *)(base + o_l0);
    ed.tri = (const int4 *)(base + o_tri);
    ed.u = S->d_u_final;
    e = cudaMemcpyAsync(S->arena, img.bytes.data(), img.bytes.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        delete S;
        return fail(NR_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
    }
    S->points = h.points;
    *out = S;
    return NR_OK;
}

int nr_spr_destroy(nr_spr *s) {
    delete s;
    return NR_OK;
}

void nr_spr_info(const nr_spr *s, nr_spr_info_t *info) {
    info->n_points = s->n;
    info->n_free_dofs = s->nr;
    info->nnz_upper = s->nnz_upper;
    info->sell_entries = s->sell_len;
    info->n_triples = s->n_triples;
    info->iterations[0] = s->iterations[0];
    info->iterations[1] = s->iterations[1];
    info->rel_residual[0] = s->rel_residual[0];
    info->rel_residual[1] = s->rel_residual[1];
    info->minx = s->minx;
    info->maxx = s->maxx;
    info->miny = s->miny;
    info->maxy = s->maxy;
}

int nr_spr_solve(nr_spr *S, int affine, double tol, int max_iter, void *stream) {
    if (!S || !(tol > 0) || max_iter < 0) return fail(NR_ERR_INVALID, "nr_spr_solve: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    S->solved_affine = -1;
    if (S->nr == 0) {
        S->solved_affine = affine ? 1 : 0;
        S->iterations[0] = S->iterations[1] = 0;
        S->rel_residual[0] = S->rel_residual[1] = 0;
        return NR_OK;
    }
    std::vector<double> rhs2, rhs_dev(2 * (size_t)S->nr);
    unit_rhs(*S, affine, rhs2);
    for (int k = 0; k < S->nr; ++k) { /* device order */
        rhs_dev[2 * (size_t)k] = rhs2[2 * (size_t)S->perm[k]];
        rhs_dev[2 * (size_t)k + 1] = rhs2[2 * (size_t)S->perm[k] + 1];
    }
    SPR_TRY(cudaMemcpyAsync((void *)S->dev.b, rhs_dev.data(), sizeof(double) * rhs_dev.size(), cudaMemcpyHostToDevice,
                            s));
    SPR_TRY(cudaStreamSynchronize(s)); /* rhs_dev is a local */
    SPR_TRY(cudaMemsetAsync(S->dev.sc, 0, sizeof(SprScal), s));
    SPR_TRY(cudaMemsetAsync(S->dev.bar, 0, sizeof(FireState), s));
    const int blocks = S->pcg_blocks;
    SprDev dd = S->dev;
    double tt = tol;
    int mi = max_iter;
    const char *env = getenv("NR_BARRIER_BUDGET_MS");
    double ms = env ? atof(env) : 2000.0;
    if (!(ms > 0)) ms = 2000.0;
    unsigned long long budget = (unsigned long long)(ms * 1e6);
    void *args[] = {&dd, &tt, &mi, &budget};
    SPR_TRY(cudaLaunchCooperativeKernel((const void *)k_spr_pcg, dim3(blocks), dim3(kSprThreads), args, 0, s));
    SprScal sc;
    FireState bar;
    SPR_TRY(cudaMemcpyAsync(&sc, S->dev.sc, sizeof(sc), cudaMemcpyDeviceToHost, s));
    SPR_TRY(cudaMemcpyAsync(&bar, S->dev.bar, sizeof(bar), cudaMemcpyDeviceToHost, s));
    SPR_TRY(cudaStreamSynchronize(s));
    if (bar.abort_flag) return fail(NR_ERR_TIMEOUT, "nr_spr_solve: grid barrier wait budget exceeded");
    for (int k = 0; k < 2; ++k) {
        S->iterations[k] = sc.iters[k];
        S->rel_residual[k] = sc.bb[k] > 0 ? std::sqrt(sc.rr[k] / sc.bb[k]) : 0.0;
        if (!std::isfinite(S->rel_residual[k])) return fail(NR_ERR_NONFINITE, "nr_spr_solve: non-finite residual");
    }
    S->solved_affine = affine ? 1 : 0;
    return (sc.active[0] || sc.active[1]) ? NR_NOT_CONVERGED : NR_OK;
}

int nr_spr_point(nr_spr *S, double compression, double shear, nr_spr_record *rec, double *u_final, void *stream) {
    if (!S || !rec) return fail(NR_ERR_INVALID, "nr_spr_point: null argument");
    if (S->solved_affine < 0) return fail(NR_ERR_INVALID, "nr_spr_point: nr_spr_solve has not run");
    cudaStream_t s = (cudaStream_t)stream;
    SprPointDev a;
    a.n = S->n;
    a.nr = S->nr;
    a.miny = S->miny;
    a.maxy = S->maxy;
    a.compression = compression;
    a.shear = shear;
    a.affine = S->solved_affine;
    a.pos = S->edev.pos;
    a.dof_map = S->d_dof_map;
    a.top = S->d_top;
    a.xsol = S->dev.x;
    a.u_red = S->d_u_red;
    a.u_final = S->d_u_final;
    k_spr_field<<<(S->n + 255) / 256, 256, 0, s>>>(a);
    SPR_TRY(cudaGetLastError());
    double resid = 0.0;
    if (S->nr > 0) {
        const int blocks = std::max(1, std::min(S->rpart_blocks, (S->n_slices + 15) / 16));
        k_spr_residual<<<blocks, kSprThreads, 0, s>>>(S->dev, S->d_u_red, compression, shear, S->d_rpart);
        k_spr_sum_parts<<<1, 32 * kParts, 0, s>>>(S->d_rpart, blocks, S->d_scalar);
        SPR_TRY(cudaGetLastError());
    }
    const int use_ss = S->ks > 0 || S->mu > 0, use_bend = S->kb > 0;
    const int tb = use_ss ? (S->n_edges + kTile - 1) / kTile : 0;
    const int tt = use_bend ? (S->n_triples + kTile - 1) / kTile : 0;
    if (tb + tt > 0)
        k_spr_energy_tiles<<<std::max(1, std::min(tb + tt, 4 * sm_count_spr())), kTile, 0, s>>>(
            S->edev, use_ss, use_bend, S->d_epart, S->e_stride);
    k_spr_energy_final<<<1, kTile, 0, s>>>(S->d_epart, tb, tt, S->e_stride, S->d_scalar + 1);
    SPR_TRY(cudaGetLastError());
    double host[3] = {0.0, 0.0, 0.0};
    SPR_TRY(cudaMemcpyAsync(host, S->d_scalar, sizeof(host), cudaMemcpyDeviceToHost, s));
    if (u_final)
        SPR_TRY(cudaMemcpyAsync(u_final, S->d_u_final, sizeof(double2) * (size_t)S->n, cudaMemcpyDefault, s));
    SPR_TRY(cudaStreamSynchronize(s));
    resid = S->nr > 0 ? std::sqrt(host[0]) : 0.0;
    rec->compression = compression;
    rec->shear = shear;
    rec->e_ss = host[1];
    rec->e_bend = host[2];
    rec->e_total = host[1] + host[2];
    rec->residual = resid;
    rec->iterations = std::max(S->iterations[0], S->iterations[1]);
    rec->status = NR_OK;
    return NR_OK;
}

}  // extern "C"
