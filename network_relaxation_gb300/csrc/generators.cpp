/*
 * Synthetic network generators.  The reference ships no inputs and no
 * generators; these produce the .dat-compatible networks the benchmarks and
 * tests run on.  Random numbers come from SplitMix64 (Steele, Lea & Flood,
 * "Fast splittable pseudorandom number generators", OOPSLA 2014), so a seed
 * fixes a network on every machine.
 *
 * Compiled with -ffp-contract=off: rest lengths must round exactly as
 * read_network computes them (large_strain_relax.cu:97-99) so a network
 * written to .dat and read back is bit-identical.
 */
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <map>
#include <vector>

#include "canon_math.h"
#include "nr_internal.h"

namespace {

struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
};

double rest_length(const std::vector<double> &p, int i1, int i2, int wrap, double offset) {
    const double dx = p[2 * i2] + offset * wrap - p[2 * i1];
    const double dy = p[2 * i2 + 1] - p[2 * i1 + 1];
    return std::sqrt(dx * dx + dy * dy);
}

/* phi0 = rest angle - pi of triple (h, j, k), computed with the same
 * canonical formula the force kernels use so the rest state is exactly
 * force-free. */
double rest_phi0(const std::vector<double> &p, int h, int j, int k, int wj, int wk, double offset) {
    const double wjW = nr::wrap_shift(wj, offset), wkW = nr::wrap_shift(wk, offset);
    const double ax = (p[2 * j] + wjW) - p[2 * h], ay = p[2 * j + 1] - p[2 * h + 1];
    const double bx = (p[2 * k] + wkW) - p[2 * h], by = p[2 * k + 1] - p[2 * h + 1];
    return nr::bend_dtheta(ax, ay, bx, by, 0.0);
}

}  // namespace

using nr::fail;

extern "C" int nr_gen_lattice(int nx, int ny, double p, double jitter, uint64_t seed, int line_triples,
                              nr_host_network **out) {
    if (!out || nx < 2 || ny < 2 || (long)nx * ny > (1L << 28) || !(p >= 0 && p <= 1) || !(jitter >= 0 && jitter < 0.25))
        return fail(NR_ERR_INVALID, "nr_gen_lattice: bad arguments");
    SplitMix64 rng(seed);
    auto *net = new nr_host_network();
    const int n = nx * ny;
    net->n_points = n;
    net->offset = nx;
    net->points.resize(2 * (size_t)n);
    const double row = std::sqrt(3.0) / 2.0;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int id = j * nx + i;
            net->points[2 * id] = i + 0.5 * (j & 1);
            net->points[2 * id + 1] = j * row;
        }
    if (jitter > 0) {
        for (int id = 0; id < n; ++id) {
            const double dx = jitter * (2.0 * rng.uniform() - 1.0);
            const double dy = jitter * (2.0 * rng.uniform() - 1.0);
            const int j = id / nx;
            net->points[2 * id] += dx;
            if (j != 0 && j != ny - 1) net->points[2 * id + 1] += dy;
        }
    }
    // Directions 0..5: right, up-right, up-left, left, down-left, down-right.
    // nbr[6*id + d] = neighbour id (or -1), nwrap = its wrap seen from id.
    std::vector<int> nbr(6 * (size_t)n, -1);
    std::vector<signed char> nwrap(6 * (size_t)n, 0);
    auto link = [&](int a, int b, int wrap, int dir) {
        net->edge_ij.push_back(a);
        net->edge_ij.push_back(b);
        net->edge_wrap.push_back((signed char)wrap);
        net->edge_l0.push_back(rest_length(net->points, a, b, wrap, net->offset));
        nbr[6 * (size_t)a + dir] = b;
        nwrap[6 * (size_t)a + dir] = (signed char)wrap;
        nbr[6 * (size_t)b + (dir + 3) % 6] = a;
        nwrap[6 * (size_t)b + (dir + 3) % 6] = (signed char)(-wrap);
    };
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int id = j * nx + i;
            // right
            {
                const double u = rng.uniform();
                const int i2 = (i + 1) % nx;
                if (u < p) link(id, j * nx + i2, i == nx - 1 ? 1 : 0, 0);
            }
            // up-left, up-right
            const bool odd = j & 1;
            {
                const double u = rng.uniform();
                if (j + 1 < ny) {
                    int i2 = odd ? i : i - 1, w = 0;
                    if (i2 < 0) { i2 += nx; w = -1; }
                    if (u < p) link(id, (j + 1) * nx + i2, w, 2);
                }
            }
            {
                const double u = rng.uniform();
                if (j + 1 < ny) {
                    int i2 = odd ? i + 1 : i, w = 0;
                    if (i2 >= nx) { i2 -= nx; w = 1; }
                    if (u < p) link(id, (j + 1) * nx + i2, w, 1);
                }
            }
        }
    nr::y_range(net->points, net->miny, net->maxy);
    if (line_triples) {
        for (int h = 0; h < n; ++h)
            for (int axis = 0; axis < 3; ++axis) {
                const int jn = nbr[6 * (size_t)h + axis + 3], kn = nbr[6 * (size_t)h + axis];
                if (jn < 0 || kn < 0) continue;
                const int wj = nwrap[6 * (size_t)h + axis + 3], wk = nwrap[6 * (size_t)h + axis];
                net->tri_hjk.push_back(h);
                net->tri_hjk.push_back(jn);
                net->tri_hjk.push_back(kn);
                net->tri_wrap.push_back((signed char)wj);
                net->tri_wrap.push_back((signed char)wk);
                net->tri_phi0.push_back(rest_phi0(net->points, h, jn, kn, wj, wk, net->offset));
            }
    }
    *out = net;
    return NR_OK;
}

namespace {

/* One straight fiber after the cut at y = 0 and y = 1: endpoints in an
 * unwrapped x frame (the periodic box is [0, 1) in x). */
struct Fiber {
    double ax, ay, bx, by;
    bool cut_a, cut_b; /* end lies on y = 0 or y = 1 (a clamped boundary node) */
};

/* Crossing of segments p + t r and q + s w (t, s in [0, 1]); false when
 * parallel or disjoint. */
bool crossing(double px, double py, double rx, double ry, double qx, double qy, double wx, double wy, double &t,
              double &s) {
    const double den = rx * wy - ry * wx;
    if (den == 0.0) return false;
    const double dx = qx - px, dy = qy - py;
    t = (dx * wy - dy * wx) / den;
    s = (dx * ry - dy * rx) / den;
    return t >= 0.0 && t <= 1.0 && s >= 0.0 && s <= 1.0;
}

double wrap01(double x) {
    double v = x - std::floor(x);
    return v >= 1.0 ? 0.0 : v;
}

}  // namespace

extern "C" int nr_gen_mikado(int n_fibers, double fiber_len, double k0, double kappa0, uint64_t seed,
                             nr_host_network **out) {
    if (!out || n_fibers <= 0 || n_fibers > (1 << 24) || !(fiber_len > 0 && fiber_len < 0.5) || !(k0 > 0) ||
        !(kappa0 >= 0))
        return fail(NR_ERR_INVALID, "nr_gen_mikado: bad arguments");
    *out = nullptr;
    SplitMix64 rng(seed);
    const double pi = 3.14159265358979323846;
    std::vector<Fiber> fib;
    fib.reserve(n_fibers);
    for (int f = 0; f < n_fibers; ++f) {
        const double cx = rng.uniform(), cy = rng.uniform(), th = pi * rng.uniform();
        const double hx = 0.5 * fiber_len * std::cos(th), hy = 0.5 * fiber_len * std::sin(th);
        Fiber g{cx - hx, cy - hy, cx + hx, cy + hy, false, false};
        /* cut at y = 0 and y = 1 */
        double t0 = 0.0, t1 = 1.0;
        const double dy = g.by - g.ay;
        if (dy != 0.0) {
            const double ta = (0.0 - g.ay) / dy, tb = (1.0 - g.ay) / dy;
            const double lo = std::min(ta, tb), hi = std::max(ta, tb);
            t0 = std::max(t0, lo);
            t1 = std::min(t1, hi);
        } else if (g.ay < 0.0 || g.ay > 1.0) {
            continue;
        }
        if (!(t1 > t0)) continue;
        const double dx = g.bx - g.ax;
        Fiber c{g.ax + t0 * dx, g.ay + t0 * dy, g.ax + t1 * dx, g.ay + t1 * dy, t0 > 0.0, t1 < 1.0};
        if (c.cut_a) c.ay = (c.ay < 0.5) ? 0.0 : 1.0;
        if (c.cut_b) c.by = (c.by < 0.5) ? 0.0 : 1.0;
        fib.push_back(c);
    }
    const int nf = (int)fib.size();
    /* nodes: position in the box and whether clamped; per fiber its nodes
     * as (t, node, unwrapped x) */
    std::vector<double> nx, ny;
    std::vector<char> boundary;
    struct Stop {
        double t;
        int node;
        double xu;
    };
    std::vector<std::vector<Stop>> stops(nf);
    auto add_node = [&](double x, double y, bool bnd) {
        nx.push_back(wrap01(x));
        ny.push_back(y);
        boundary.push_back(bnd ? 1 : 0);
        return (int)nx.size() - 1;
    };
    for (int f = 0; f < nf; ++f) {
        const Fiber &c = fib[f];
        if (c.cut_a) stops[f].push_back({0.0, add_node(c.ax, c.ay, true), c.ax});
        if (c.cut_b) stops[f].push_back({1.0, add_node(c.bx, c.by, true), c.bx});
    }
    /* crossings: a uniform grid of cells at least one fiber long; a pair is
     * tested in every cell both touch and kept only in the cell holding the
     * crossing point */
    const int ncx = std::max(1, (int)std::floor(1.0 / fiber_len)), ncy = ncx;
    std::vector<std::vector<int>> cell((size_t)ncx * ncy);
    auto cx_of = [&](double x) { return std::min(ncx - 1, (int)(wrap01(x) * ncx)); };
    auto cy_of = [&](double y) { return std::min(ncy - 1, std::max(0, (int)(y * ncy))); };
    for (int f = 0; f < nf; ++f) {
        const Fiber &c = fib[f];
        const double x0 = std::min(c.ax, c.bx), x1 = std::max(c.ax, c.bx);
        const double y0 = std::min(c.ay, c.by), y1 = std::max(c.ay, c.by);
        const int i0 = (int)std::floor(x0 * ncx), i1 = (int)std::floor(x1 * ncx);
        const int j0 = cy_of(y0), j1 = cy_of(y1);
        for (int i = i0; i <= i1; ++i)
            for (int j = j0; j <= j1; ++j) cell[(size_t)(((i % ncx) + ncx) % ncx) * ncy + j].push_back(f);
    }
    for (int ci = 0; ci < ncx; ++ci)
        for (int cj = 0; cj < ncy; ++cj) {
            const std::vector<int> &lst = cell[(size_t)ci * ncy + cj];
            for (size_t a = 0; a < lst.size(); ++a)
                for (size_t b = a + 1; b < lst.size(); ++b) {
                    const int f = std::min(lst[a], lst[b]), g = std::max(lst[a], lst[b]);
                    if (f == g) continue;
                    const Fiber &F = fib[f], &G = fib[g];
                    for (int sh = -1; sh <= 1; ++sh) {
                        double t, s;
                        if (!crossing(F.ax, F.ay, F.bx - F.ax, F.by - F.ay, G.ax + sh, G.ay, G.bx - G.ax, G.by - G.ay,
                                      t, s))
                            continue;
                        const double px = F.ax + t * (F.bx - F.ax), py = F.ay + t * (F.by - F.ay);
                        if (cx_of(px) != ci || cy_of(py) != cj) break;
                        const int node = add_node(px, py, false);
                        stops[f].push_back({t, node, px});
                        stops[g].push_back({s, node, px - sh});
                        break;
                    }
                }
        }
    /* segments between consecutive stops; dangling ends pruned repeatedly */
    struct Seg {
        int a, b, fiber;
        double dxu, dyu; /* b - a in the fiber's unwrapped frame */
    };
    std::vector<Seg> seg;
    for (int f = 0; f < nf; ++f) {
        std::vector<Stop> &st = stops[f];
        std::sort(st.begin(), st.end(), [](const Stop &x, const Stop &y) { return x.t < y.t; });
        for (size_t k = 1; k < st.size(); ++k)
            seg.push_back({st[k - 1].node, st[k].node, f, st[k].xu - st[k - 1].xu, ny[st[k].node] - ny[st[k - 1].node]});
    }
    const int nn = (int)nx.size();
    std::vector<std::vector<int>> adj(nn);
    for (int e = 0; e < (int)seg.size(); ++e) {
        adj[seg[e].a].push_back(e);
        adj[seg[e].b].push_back(e);
    }
    std::vector<char> seg_alive(seg.size(), 1), node_alive(nn, 1);
    std::vector<int> deg(nn);
    std::vector<int> work;
    for (int v = 0; v < nn; ++v) {
        deg[v] = (int)adj[v].size();
        if (deg[v] == 0 || (deg[v] == 1 && !boundary[v])) work.push_back(v);
    }
    while (!work.empty()) {
        const int v = work.back();
        work.pop_back();
        if (!node_alive[v]) continue;
        node_alive[v] = 0;
        for (int e : adj[v]) {
            if (!seg_alive[e]) continue;
            seg_alive[e] = 0;
            const int o = seg[e].a == v ? seg[e].b : seg[e].a;
            if (--deg[o] == 0 || (deg[o] == 1 && !boundary[o])) work.push_back(o);
        }
    }
    /* renumber the surviving nodes by y (then x): consecutive node blocks are
     * horizontal bands */
    std::vector<int> keep;
    for (int v = 0; v < nn; ++v)
        if (node_alive[v]) keep.push_back(v);
    std::stable_sort(keep.begin(), keep.end(), [&](int a, int b) { return ny[a] < ny[b] || (ny[a] == ny[b] && nx[a] < nx[b]); });
    if (keep.empty()) return fail(NR_ERR_INVALID, "nr_gen_mikado: no connected network (too few fibers)");
    std::vector<int> id(nn, -1);
    auto *net = new nr_host_network();
    net->n_points = (int)keep.size();
    net->offset = 1.0;
    net->points.resize(2 * keep.size());
    for (size_t k = 0; k < keep.size(); ++k) {
        id[keep[k]] = (int)k;
        net->points[2 * k] = nx[keep[k]];
        net->points[2 * k + 1] = ny[keep[k]];
    }
    auto wrap_of = [&](int i1, int i2, double dxu) {
        return (int)std::lround(dxu - (net->points[2 * i2] - net->points[2 * i1]));
    };
    std::vector<int> seg_bond(seg.size(), -1);
    for (size_t e = 0; e < seg.size(); ++e) {
        if (!seg_alive[e]) continue;
        const int i1 = id[seg[e].a], i2 = id[seg[e].b];
        const int w = wrap_of(i1, i2, seg[e].dxu);
        seg_bond[e] = net->n_edges();
        net->edge_ij.push_back(i1);
        net->edge_ij.push_back(i2);
        net->edge_wrap.push_back((signed char)w);
        const double l0 = rest_length(net->points, i1, i2, w, 1.0);
        net->edge_l0.push_back(l0);
        net->bond_k.push_back(k0 / l0);
    }
    /* triples: consecutive surviving segments of a fiber */
    for (size_t e = 1; e < seg.size(); ++e) {
        const Seg &s1 = seg[e - 1], &s2 = seg[e];
        if (s1.fiber != s2.fiber || !seg_alive[e - 1] || !seg_alive[e] || s1.b != s2.a) continue;
        const int h = id[s1.b], j = id[s1.a], k = id[s2.b];
        const int wj = wrap_of(h, j, -s1.dxu), wk = wrap_of(h, k, s2.dxu);
        net->tri_hjk.push_back(h);
        net->tri_hjk.push_back(j);
        net->tri_hjk.push_back(k);
        net->tri_wrap.push_back((signed char)wj);
        net->tri_wrap.push_back((signed char)wk);
        const double lbar = 0.5 * (net->edge_l0[seg_bond[e - 1]] + net->edge_l0[seg_bond[e]]);
        net->tri_kb.push_back(kappa0 / lbar);
        net->tri_phi0.push_back(rest_phi0(net->points, h, j, k, wj, wk, 1.0));
    }
    nr::y_range(net->points, net->miny, net->maxy);
    *out = net;
    return NR_OK;
}

/* Fiber network embedded in a gel, the input of network_mesh_relax.cu (the
 * reference ships no such files).  Nodes on an nx x ny unit grid plus a copy
 * of column 0 at x = nx, the mesh's right edge, which the reader's
 * duplicate-vertex search pairs with column 0.  Every grid cell is split
 * along its up-right diagonal into two gel triangles; their areas are
 * computed from the positions.  The network lives on columns 0..nx-1: bonds
 * right (wrapping from nx-1 to 0), up and up-right, each kept with
 * probability p; the copied column carries gel only.  jitter moves interior
 * nodes by U(-jitter, jitter) in x and y; column 0 (and its copy) moves in
 * y only, and the top and bottom rows move in x only. */
extern "C" int nr_gen_lattice_mesh(int nx, int ny, double p, double jitter, uint64_t seed, nr_host_network **out) {
    if (!out || nx < 2 || ny < 2 || (long)(nx + 1) * ny > (1L << 28) || !(p >= 0 && p <= 1) ||
        !(jitter >= 0 && jitter < 0.25))
        return fail(NR_ERR_INVALID, "nr_gen_lattice_mesh: bad arguments");
    SplitMix64 rng(seed);
    const int W = nx + 1;
    auto id = [W](int i, int j) { return j * W + i; };
    auto *net = new nr_host_network();
    net->n_points = W * ny;
    net->offset = nx;
    net->points.resize(2 * (size_t)net->n_points);
    std::vector<double> &pt = net->points;
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const double dx = jitter * (2.0 * rng.uniform() - 1.0);
            const double dy = jitter * (2.0 * rng.uniform() - 1.0);
            pt[2 * id(i, j)] = i + (i == 0 ? 0.0 : dx);
            pt[2 * id(i, j) + 1] = j + (j == 0 || j == ny - 1 ? 0.0 : dy);
        }
    for (int j = 0; j < ny; ++j) {
        pt[2 * id(nx, j)] = pt[2 * id(0, j)] + nx;
        pt[2 * id(nx, j) + 1] = pt[2 * id(0, j) + 1];
    }
    auto link = [&](int a, int b, int wrap) {
        net->edge_ij.push_back(a);
        net->edge_ij.push_back(b);
        net->edge_wrap.push_back((signed char)wrap);
        net->edge_l0.push_back(rest_length(pt, a, b, wrap, net->offset));
    };
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const bool last = i == nx - 1;
            const int right = last ? 0 : i + 1;
            if (rng.uniform() < p) link(id(i, j), id(right, j), last ? 1 : 0);
            const double u_up = rng.uniform(), u_diag = rng.uniform();
            if (j + 1 < ny) {
                if (u_up < p) link(id(i, j), id(i, j + 1), 0);
                if (u_diag < p) link(id(i, j), id(right, j + 1), last ? 1 : 0);
            }
        }
    auto area = [&](int a, int b, int c) {
        const double ux = pt[2 * b] - pt[2 * a], uy = pt[2 * b + 1] - pt[2 * a + 1];
        const double vx = pt[2 * c] - pt[2 * a], vy = pt[2 * c + 1] - pt[2 * a + 1];
        return 0.5 * std::fabs(ux * vy - uy * vx);
    };
    for (int j = 0; j + 1 < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            const int a = id(i, j), b = id(i + 1, j), c = id(i, j + 1), d = id(i + 1, j + 1);
            const int tris[2][3] = {{a, b, d}, {a, d, c}};
            for (const auto &t : tris) {
                net->facets.insert(net->facets.end(), t, t + 3);
                net->areas.push_back(area(t[0], t[1], t[2]));
            }
        }
    nr::y_range(pt, net->miny, net->maxy);
    net->minx = FLT_MAX;
    net->maxx = FLT_MIN;
    for (int v = 0; v < net->n_points; ++v) {
        net->minx = std::min(net->minx, pt[2 * v]);
        net->maxx = std::max(net->maxx, pt[2 * v]);
    }
    nr::find_mesh_pairs(pt, net->offset, net->minx, net->mesh_pairs);
    *out = net;
    return NR_OK;
}
