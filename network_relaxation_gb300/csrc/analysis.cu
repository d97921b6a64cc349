/*
 * Post-relaxation analyses on the GPU: the computations of the reference's
 * analysis programs, on reference positions and a displacement field.
 *
 *   nr_bond_strains          strain_calc.cpp:96-120 (get_strains)
 *   nr_linear_axial_energy   axial_contribution.cpp:64-70, 176-190
 *   nr_nonaffinity           na_calc.cpp:308-327 (calc_na_val)
 *
 * Per-item arithmetic follows the reference operation for operation
 * (compiled with --fmad=false, so products and sums round as written);
 * the totals use the canonical reduction tree of nr_device.cuh (tiles of
 * 256, warp butterflies, tree of 8, per-lane tile accumulation) instead of
 * the reference's sequential loops, so they are reproducible and equal the
 * oracle's or_canon_sum bit for bit.
 *
 * Arrays may be host or device memory: inputs that are not device memory
 * are staged into device buffers, outputs are copied to wherever they
 * point (cudaMemcpyDefault); the calls return after the stream finishes.
 */
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "nr_device.cuh"
#include "nr_internal.h"

namespace nr {
namespace {

struct EdgeIn {
    int n_edges;
    double width;
    const int *ij;
    const signed char *wrap;
    const double *pos0, *disp;
};

__device__ __forceinline__ double bond_strain(const EdgeIn &a, int b) {
    const int i1 = a.ij[2 * b], i2 = a.ij[2 * b + 1];
    const double dxi = a.pos0[2 * i2] + a.wrap[b] * a.width - a.pos0[2 * i1];
    const double dyi = a.pos0[2 * i2 + 1] - a.pos0[2 * i1 + 1];
    const double dxf = dxi + a.disp[2 * i2] - a.disp[2 * i1];
    const double dyf = dyi + a.disp[2 * i2 + 1] - a.disp[2 * i1 + 1];
    const double li = sqrt(dxi * dxi + dyi * dyi);
    const double lf = sqrt(dxf * dxf + dyf * dyf);
    return (lf - li) / li;
}

__device__ __forceinline__ double axial_term(const EdgeIn &a, int b) {
    const int i1 = a.ij[2 * b], i2 = a.ij[2 * b + 1];
    double dx = a.pos0[2 * i2] + a.width * a.wrap[b] - a.pos0[2 * i1];
    double dy = a.pos0[2 * i2 + 1] - a.pos0[2 * i1 + 1];
    const double length = sqrt(dx * dx + dy * dy);
    dx /= length;
    dy /= length;
    const double proj = (a.disp[2 * i2] - a.disp[2 * i1]) * dx + (a.disp[2 * i2 + 1] - a.disp[2 * i1 + 1]) * dy;
    return .5 * proj * proj;
}

struct NodeIn {
    int n_points;
    double miny, axial, shear;
    const double *pos0, *disp;
};

__device__ __forceinline__ double na_term(const NodeIn &a, int i) {
    const double y = a.pos0[2 * i + 1];
    const double ux_a = a.disp[2 * i], uy_a = a.disp[2 * i + 1];
    const double ux_e = (y - a.miny) * a.shear, uy_e = (y - a.miny) * a.axial;
    return (ux_a - ux_e) * (ux_a - ux_e) + (uy_a - uy_e) * (uy_a - uy_e);
}

__global__ void k_bond_strains(EdgeIn a, double *out) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < a.n_edges; b += gridDim.x * blockDim.x)
        out[b] = bond_strain(a, b);
}

/* Tile partials of the canonical sum of term(i), i < n; one tile of 256
 * items per CTA iteration. */
template <class In, double (*Term)(const In &, int)>
__global__ void __launch_bounds__(kTile) k_tile_sums(In a, int n, double *partials) {
    __shared__ double s_red[kTile / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tiles = (n + kTile - 1) / kTile;
    for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
        const int i = t * kTile + threadIdx.x;
        double e = i < n ? Term(a, i) : 0.0;
        e = warp_sum(e);
        if (lane == 0) s_red[warp] = e;
        __syncthreads();
        if (threadIdx.x == 0) partials[t] = tree8(s_red);
        __syncthreads();
    }
}

/* out = (canonical sum of the tile partials) * scale, or / divisor. */
__global__ void __launch_bounds__(kTile) k_final(const double *partials, int tiles, double scale, double divisor,
                                                 double *out) {
    __shared__ double s_red[kTile / 32];
    const double s = tiles > 0 ? final_sum(partials, tiles, 8, s_red) : 0.0;
    if (threadIdx.x == 0) out[0] = divisor != 0.0 ? s / divisor : s * scale;
}

/* A device view of a caller array: the array itself when the device can
 * address it, else a device copy.  Scratch comes from the stream-ordered
 * pool allocator (cudaMallocAsync / cudaFreeAsync on the call's stream):
 * no device-wide synchronisation and no allocation cost after the pool
 * has warmed up. */
struct Staged {
    const void *dev = nullptr;
    void *own = nullptr;
    cudaStream_t stream = nullptr;
    ~Staged() {
        if (own) cudaFreeAsync(own, stream);
    }
};

/* The library's own stream-ordered pool on the current device, created on
 * first use, whose release threshold keeps its memory mapped between calls
 * (the default pool returns it at every synchronisation, and mapping it
 * again costs more than the analyses themselves).  It holds at most the
 * largest scratch the analyses have needed, for the life of the process.
 * nullptr if pools are unsupported. */
cudaMemPool_t scratch_pool() {
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lock(mu);
    auto it = pools.find(dev);
    if (it != pools.end()) return it->second;
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
        cudaGetLastError();
        pool = nullptr;
    } else {
        cuuint64_t keep = ~(cuuint64_t)0;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    pools[dev] = pool;
    return pool;
}

cudaError_t scratch_alloc(Staged &st, size_t bytes, cudaStream_t s) {
    st.stream = s;
    cudaMemPool_t pool = scratch_pool();
    cudaError_t e = pool ? cudaMallocFromPoolAsync(&st.own, bytes, pool, s) : cudaMallocAsync(&st.own, bytes, s);
    if (e != cudaSuccess) st.own = nullptr;
    return e;
}

bool device_accessible(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int stage(const void *src, size_t bytes, cudaStream_t s, Staged &st) {
    if (!src || bytes == 0) {
        st.dev = src;
        return NR_OK;
    }
    if (device_accessible(src)) {
        st.dev = src;
        return NR_OK;
    }
    cudaError_t e = scratch_alloc(st, bytes, s);
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? NR_ERR_OOM : NR_ERR_CUDA,
                    std::string("analysis: cudaMallocAsync: ") + cudaGetErrorString(e));
    e = cudaMemcpyAsync(st.own, src, bytes, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return fail(NR_ERR_CUDA, std::string("analysis: copy: ") + cudaGetErrorString(e));
    st.dev = st.own;
    return NR_OK;
}

int sms() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

/* Canonical sum of Term over n items into *out (host or device). */
template <class In, double (*Term)(const In &, int)>
int canonical_total(const In &a, int n, double scale, double divisor, double *out, cudaStream_t s) {
    const int tiles = (n + kTile - 1) / kTile;
    Staged part;
    cudaError_t e = scratch_alloc(part, sizeof(double) * (size_t)(tiles > 0 ? tiles : 1) + sizeof(double), s);
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? NR_ERR_OOM : NR_ERR_CUDA,
                    std::string("analysis: cudaMallocAsync: ") + cudaGetErrorString(e));
    double *partials = (double *)part.own, *total = partials + (tiles > 0 ? tiles : 1);
    if (tiles > 0) k_tile_sums<In, Term><<<std::min(tiles, 8 * sms()), kTile, 0, s>>>(a, n, partials);
    k_final<<<1, kTile, 0, s>>>(partials, tiles, scale, divisor, total);
    if ((e = cudaGetLastError()) != cudaSuccess)
        return fail(NR_ERR_CUDA, std::string("analysis: launch: ") + cudaGetErrorString(e));
    if ((e = cudaMemcpyAsync(out, total, sizeof(double), cudaMemcpyDefault, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return fail(NR_ERR_CUDA, std::string("analysis: ") + cudaGetErrorString(e));
    return NR_OK;
}

int check_edges(int n_points, int n_edges, const double *pos0, const double *disp, const int *ij,
                const signed char *wrap) {
    if (n_points <= 0 || n_edges < 0) return fail(NR_ERR_INVALID, "analysis: bad sizes");
    if (!pos0 || !disp || (n_edges > 0 && (!ij || !wrap))) return fail(NR_ERR_INVALID, "analysis: null array");
    return NR_OK;
}

}  // namespace
}  // namespace nr

using namespace nr;

extern "C" int nr_bond_strains(int n_points, int npairs, double width, const double *pos0, const double *disp,
                               const int *pair_list, const signed char *e_offsets, double *strains, void *stream) {
    clear_error();
    int st = check_edges(n_points, npairs, pos0, disp, pair_list, e_offsets);
    if (st != NR_OK) return st;
    if (!strains) return fail(NR_ERR_INVALID, "nr_bond_strains: null output");
    if (npairs == 0) return NR_OK;
    const cudaStream_t s = (cudaStream_t)stream;
    Staged p0, u, ij, w, out;
    if ((st = stage(pos0, sizeof(double) * 2 * (size_t)n_points, s, p0)) != NR_OK) return st;
    if ((st = stage(disp, sizeof(double) * 2 * (size_t)n_points, s, u)) != NR_OK) return st;
    if ((st = stage(pair_list, sizeof(int) * 2 * (size_t)npairs, s, ij)) != NR_OK) return st;
    if ((st = stage(e_offsets, (size_t)npairs, s, w)) != NR_OK) return st;
    double *dout = strains;
    if (!device_accessible(strains)) {
        cudaError_t e = scratch_alloc(out, sizeof(double) * (size_t)npairs, s);
        if (e != cudaSuccess)
            return fail(NR_ERR_OOM, std::string("nr_bond_strains: cudaMallocAsync: ") + cudaGetErrorString(e));
        dout = (double *)out.own;
    }
    const EdgeIn a{npairs, width, (const int *)ij.dev, (const signed char *)w.dev, (const double *)p0.dev,
                   (const double *)u.dev};
    k_bond_strains<<<std::min((npairs + 255) / 256, 8 * sms()), 256, 0, s>>>(a, dout);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && dout != strains)
        e = cudaMemcpyAsync(strains, dout, sizeof(double) * (size_t)npairs, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(NR_ERR_CUDA, std::string("nr_bond_strains: ") + cudaGetErrorString(e));
    return NR_OK;
}

extern "C" int nr_linear_axial_energy(int n_points, int npairs, double width, double k, const double *pos0,
                                      const double *disp, const int *pair_list, const signed char *e_offsets,
                                      double *energy, void *stream) {
    clear_error();
    int st = check_edges(n_points, npairs, pos0, disp, pair_list, e_offsets);
    if (st != NR_OK) return st;
    if (!energy) return fail(NR_ERR_INVALID, "nr_linear_axial_energy: null output");
    const cudaStream_t s = (cudaStream_t)stream;
    Staged p0, u, ij, w;
    if ((st = stage(pos0, sizeof(double) * 2 * (size_t)n_points, s, p0)) != NR_OK) return st;
    if ((st = stage(disp, sizeof(double) * 2 * (size_t)n_points, s, u)) != NR_OK) return st;
    if ((st = stage(pair_list, sizeof(int) * 2 * (size_t)npairs, s, ij)) != NR_OK) return st;
    if ((st = stage(e_offsets, (size_t)npairs, s, w)) != NR_OK) return st;
    const EdgeIn a{npairs, width, (const int *)ij.dev, (const signed char *)w.dev, (const double *)p0.dev,
                   (const double *)u.dev};
    return canonical_total<EdgeIn, axial_term>(a, npairs, k, 0.0, energy, s);
}

extern "C" int nr_nonaffinity(int n_points, const double *pos0, const double *disp, double miny, double axial_strain,
                              double shear_strain, double *na, void *stream) {
    clear_error();
    if (n_points <= 0 || !pos0 || !disp || !na) return fail(NR_ERR_INVALID, "nr_nonaffinity: bad arguments");
    const cudaStream_t s = (cudaStream_t)stream;
    Staged p0, u;
    int st;
    if ((st = stage(pos0, sizeof(double) * 2 * (size_t)n_points, s, p0)) != NR_OK) return st;
    if ((st = stage(disp, sizeof(double) * 2 * (size_t)n_points, s, u)) != NR_OK) return st;
    const NodeIn a{n_points, miny, axial_strain, shear_strain, (const double *)p0.dev, (const double *)u.dev};
    return canonical_total<NodeIn, na_term>(a, n_points, 1.0, (double)n_points, na, s);
}
