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
