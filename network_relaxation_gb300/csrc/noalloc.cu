/*
 * nr_energies_noalloc: stretch and bend energies without allocating.
 *
 * Some callers cannot call cudaMalloc or cudaFree: a host framework that
 * hands all device memory out of its own pool and forbids other
 * allocations, or a tight loop that must not pay for them (both calls can
 * synchronize the whole device).  This entry point serves them.  It is the
 * canonical energy reduction of nr_energies (fire_common.cuh energy_tiles /
 * energy_final: 256-item tiles, warp butterflies, tree of 8, per-lane tile
 * accumulation), reading the network from the reference's device arrays
 * (the ones nr_run_fire_md takes) and keeping its only scratch, the
 * per-tile partial sums, in the fixed array below instead of in memory it
 * allocates.  The results are bit-identical to nr_energies on the same
 * network.
 *
 * The array lives in the library's device image: every GPU that loads the
 * library holds its 256 KiB until the process exits.  Every call shares
 * it, so calls that overlap on the GPU race: issue every call on one
 * stream, or order calls on different streams with events.  Each call writes
 * every partial its final pass reads before reading it, so nothing has to
 * start at zero and nothing is cleared.
 */
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "canon_math.h"
#include "nr_device.cuh"
#include "nr_internal.h"

namespace nr {
namespace {

constexpr int kMaxTiles = NR_NOALLOC_MAX_ITEMS / kTile;
static_assert(NR_NOALLOC_MAX_ITEMS % kTile == 0, "capacity is a whole number of tiles");

/* Tile partials: bond tiles at [0, kMaxTiles), triple tiles after them. */
static __device__ __align__(256) double g_energy_scratch[2 * kMaxTiles];

struct RefNet {
    int n_points, npairs, ntriples, use_bonds, use_triples;
    double width, ks, kb;
    const double *pos;
    const int *pairs;
    const double *lengths;
    const signed char *e_off;
    const int *triples;
    const signed char *t_off;
};

__device__ __forceinline__ bool in_range(int i, int n) { return i >= 0 && i < n; }

/* One 256-item tile per CTA iteration; an index outside [0, n_points)
 * turns the item's energy into NaN instead of reading out of bounds. */
__global__ void __launch_bounds__(kTile) k_noalloc_energy_tiles(RefNet v, double *scratch) {
    __shared__ double s_red[kTile / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tb = v.use_bonds ? (v.npairs + kTile - 1) / kTile : 0;
    const int tt = v.use_triples ? (v.ntriples + kTile - 1) / kTile : 0;
    for (int t = blockIdx.x; t < tb + tt; t += gridDim.x) {
        const bool is_bond = t < tb;
        const int tile = is_bond ? t : t - tb;
        const int item = tile * kTile + threadIdx.x;
        double e = 0.0;
        if (is_bond) {
            if (item < v.npairs) {
                const int i = v.pairs[2 * item], j = v.pairs[2 * item + 1];
                if (in_range(i, v.n_points) && in_range(j, v.n_points))
                    e = bond_energy(v.pos[2 * i], v.pos[2 * i + 1], v.pos[2 * j], v.pos[2 * j + 1],
                                    wrap_shift(v.e_off[item], v.width), v.lengths[item], v.ks);
                else
                    e = __longlong_as_double(0x7ff8000000000000LL);
            }
        } else if (item < v.ntriples) {
            const int h = v.triples[3 * item], j = v.triples[3 * item + 1], k = v.triples[3 * item + 2];
            if (in_range(h, v.n_points) && in_range(j, v.n_points) && in_range(k, v.n_points)) {
                const double W = v.width;
                const double ax = (v.pos[2 * j] + wrap_shift(v.t_off[2 * item], W)) - v.pos[2 * h];
                const double ay = v.pos[2 * j + 1] - v.pos[2 * h + 1];
                const double bx = (v.pos[2 * k] + wrap_shift(v.t_off[2 * item + 1], W)) - v.pos[2 * h];
                const double by = v.pos[2 * k + 1] - v.pos[2 * h + 1];
                e = bend_energy(ax, ay, bx, by, v.kb, 0.0);
            } else {
                e = __longlong_as_double(0x7ff8000000000000LL);
            }
        }
        e = warp_sum(e);
        if (lane == 0) s_red[warp] = e;
        __syncthreads();
        if (threadIdx.x == 0) scratch[(is_bond ? 0 : kMaxTiles) + tile] = tree8(s_red);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kTile) k_noalloc_energy_final(RefNet v, const double *scratch, double *out) {
    __shared__ double s_red[kTile / 32];
    const int tb = (v.npairs + kTile - 1) / kTile, tt = (v.ntriples + kTile - 1) / kTile;
    double es = 0.0, eb = 0.0;
    if (v.use_bonds && v.npairs > 0) es = final_sum(scratch, tb, 8, s_red);
    if (v.use_triples && v.ntriples > 0) eb = final_sum(scratch + kMaxTiles, tt, 8, s_red);
    if (threadIdx.x == 0) {
        out[0] = es;
        out[1] = eb;
    }
}

/* Device address of g_energy_scratch on the current device.  The symbol's
 * host-side name is not a device address, so it is looked up with
 * cudaGetSymbolAddress on every call: the lookup is cheap once the module is
 * loaded, and a fresh lookup stays right after cudaDeviceReset or after the
 * primary context was released and retained again, when the module may load
 * at another address.  The first lookup on a device can load the library's
 * device code, which is why the first call must come before any stream
 * capture.  Only the SM count is cached. */
constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
int g_sm_count[kMaxDevices];

int scratch_for_current_device(double **ptr, int *sms) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(NR_ERR_CUDA, std::string("nr_energies_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(NR_ERR_CAPACITY, "nr_energies_noalloc: device ordinal beyond 63");
    double *p = nullptr;
    e = cudaGetSymbolAddress((void **)&p, g_energy_scratch);
    if (e != cudaSuccess)
        return fail(NR_ERR_CUDA, std::string("nr_energies_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (g_sm_count[dev] <= 0) {
        int n = 0;
        e = cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess)
            return fail(NR_ERR_CUDA, std::string("nr_energies_noalloc: cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
        g_sm_count[dev] = n > 0 ? n : 1;
    }
    *ptr = p;
    *sms = g_sm_count[dev];
    return NR_OK;
}

}  // namespace
}  // namespace nr

extern "C" int nr_energies_noalloc(int n_points, int npairs, int ntriples, double width, double ks, double kb,
                                   const double *d_pos, const int *d_pair_list, const double *d_lengths,
                                   const signed char *d_e_offsets, const int *d_triples,
                                   const signed char *d_t_offsets, double *d_energies, void *stream) {
    using namespace nr;
    clear_error();
    if (n_points <= 0 || npairs < 0 || ntriples < 0)
        return fail(NR_ERR_INVALID, "nr_energies_noalloc: n_points must be positive, npairs and ntriples >= 0");
    if (npairs > NR_NOALLOC_MAX_ITEMS || ntriples > NR_NOALLOC_MAX_ITEMS)
        return fail(NR_ERR_CAPACITY, "nr_energies_noalloc: " + std::to_string(npairs) + " bonds / " +
                                         std::to_string(ntriples) + " triples exceed the fixed capacity of " +
                                         std::to_string(NR_NOALLOC_MAX_ITEMS) + " items each");
    RefNet v;
    v.n_points = n_points;
    v.npairs = npairs;
    v.ntriples = ntriples;
    v.use_bonds = ks > 0 && npairs > 0;
    v.use_triples = kb > 0 && ntriples > 0;
    v.width = width;
    v.ks = ks;
    v.kb = kb;
    v.pos = d_pos;
    v.pairs = d_pair_list;
    v.lengths = d_lengths;
    v.e_off = d_e_offsets;
    v.triples = d_triples;
    v.t_off = d_t_offsets;
    if (!d_energies || ((v.use_bonds || v.use_triples) && !d_pos) ||
        (v.use_bonds && (!d_pair_list || !d_lengths || !d_e_offsets)) ||
        (v.use_triples && (!d_triples || !d_t_offsets)))
        return fail(NR_ERR_INVALID, "nr_energies_noalloc: null device array");
    double *scratch = nullptr;
    int sms = 1;
    const int st = scratch_for_current_device(&scratch, &sms);
    if (st != NR_OK) return st;
    const cudaStream_t s = (cudaStream_t)stream;
    const int tiles = (v.use_bonds ? (npairs + kTile - 1) / kTile : 0) + (v.use_triples ? (ntriples + kTile - 1) / kTile : 0);
    const int blocks = tiles < 8 * sms ? (tiles > 0 ? tiles : 1) : 8 * sms;
    k_noalloc_energy_tiles<<<blocks, kTile, 0, s>>>(v, scratch);
    k_noalloc_energy_final<<<1, kTile, 0, s>>>(v, scratch, d_energies);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(NR_ERR_CUDA, std::string("nr_energies_noalloc: launch: ") + cudaGetErrorString(e));
    return NR_OK;
}
