/*
 * Plain FP64 FIRE on sm_103a: the drop-in for run_fire_md
 * (large_strain_relax.cu:596-762) with axial_forces / bending_forces
 * (:386-469) fused into a deterministic per-node gather.
 *
 * Compiled with --fmad=false: every fused multiply-add is an explicit fma()
 * in canon_math.h or below, so results are bit-identical to the CPU oracle.
 *
 * One FIRE iteration is three passes:
 *   pass A  (nodes) v mixing / zeroing from the previous step's scalars,
 *           then drift x += dt v; x += dt^2/2m F; half kick v += dt/2m F
 *   items   (bonds, triples) each force computed once into scratch
 *   pass B  (nodes) canonical-order gather of the item forces, half kick,
 *           per-node terms of P = v.F, |v|^2, |F|^2, max|F|^2 -> canonical
 *           unit partials
 * separated by barriers; after pass B one CTA finishes the reductions and
 * advances the FIRE scalars (dt, alpha, N+, convergence).  Two kernels share
 * this code:
 *   k_fire_grid   one network over many CTAs (cooperative launch, software
 *                 grid barrier with a wait budget -> NR_ERR_TIMEOUT);
 *   k_fire_batch  many networks, one CTA per network, persistent over a
 *                 device work queue; __syncthreads only.
 */
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "fire_common.cuh"
#include "fire_launch.h"

namespace nr {

/* Pass A of node i: mixing / zeroing from the previous step's scalars,
 * drift, half kick. */
__device__ __forceinline__ void pass_a_node(const NetDev &d, const Scal &s, int i) {
    double2 xi = d.x[i], vi = d.v[i];
    const double2 fi = d.f[i];
    if (s.mix_pending) {
        vi.x = fma(s.mix_na, vi.x, vi.x);
        vi.y = fma(s.mix_na, vi.y, vi.y);
        vi.x = fma(s.mix_a, fi.x, vi.x);
        vi.y = fma(s.mix_a, fi.y, vi.y);
        if (s.zero_v) vi = make_double2(0.0, 0.0);
    }
    if (!s.done) {
        xi.x = fma(s.dt, vi.x, xi.x);
        xi.y = fma(s.dt, vi.y, xi.y);
        xi.x = fma(s.dtsq, fi.x, xi.x);
        xi.y = fma(s.dtsq, fi.y, xi.y);
        vi.x = fma(s.dtm, fi.x, vi.x);
        vi.y = fma(s.dtm, fi.y, vi.y);
        d.x[i] = xi;
    }
    d.v[i] = vi;
}

/* Pass A over the nodes of units u = u0, u0+ustride, ... */
__device__ void pass_a(const NetDev &d, const Scal &s, int u0, int ustride) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int u = u0; u < d.n_units; u += ustride) {
        const int i = (u * d.sub + warp) * kChunk + lane;
        if (i >= d.n) continue;
        pass_a_node(d, s, i);
    }
}

/* Pass B: forces at the current x, half kick (or v = 0 when init), and the
 * canonical unit partials of P, |v|^2, |F|^2, max|F|^2 into d.part. */
template <bool kGel>
__device__ void pass_b(const NetDev &d, double dtm, bool init, int u0, int ustride, double *s_units) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, sub = d.sub;
    for (int ubase = u0; ubase < d.n_units; ubase += ustride * kGroup) {
        int gn = 0;
        for (int u = ubase; u < d.n_units && gn < kGroup; u += ustride, ++gn) {
            const int i = (u * sub + warp) * kChunk + lane;
            double tP = 0.0, tV = 0.0, tF = 0.0;
            if (i < d.n) {
                double fx, fy;
                node_force_items<kGel>(d, i, fx, fy);
                double2 vi;
                if (init) {
                    vi = make_double2(0.0, 0.0);
                } else {
                    vi = d.v[i];
                    vi.x = fma(dtm, fx, vi.x);
                    vi.y = fma(dtm, fy, vi.y);
                }
                d.v[i] = vi;
                d.f[i] = make_double2(fx, fy);
                tP = dot2(vi.x, vi.y, fx, fy);
                tV = dot2(vi.x, vi.y, vi.x, vi.y);
                tF = dot2(fx, fy, fx, fy);
            }
            const double sP = warp_sum(tP), sV = warp_sum(tV), sF = warp_sum(tF), sM = warp_max(tF);
            if (lane == 0) {
                double *w = s_units + (size_t)gn * 4 * sub;
                w[0 * sub + warp] = sP;
                w[1 * sub + warp] = sV;
                w[2 * sub + warp] = sF;
                w[3 * sub + warp] = sM;
            }
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < gn * 4; idx += blockDim.x) {
            const int g = idx >> 2, q = idx & 3;
            const int u = ubase + g * ustride;
            const double *w = s_units + (size_t)g * 4 * sub + q * sub;
            double val;
            if (q < 3) {
                val = subtree(w, sub);
            } else {
                val = w[0];
                for (int k = 1; k < sub; ++k) val = fmax(val, w[k]);
            }
            d.part[(size_t)q * d.n_units + u] = val;
        }
        __syncthreads();
    }
}

/* Final reductions of d.part by the calling CTA (all threads get them). */
__device__ void reduce_parts(const NetDev &d, double *s_red, double &P, double &V2, double &F2, double &M2) {
    P = final_sum(d.part, d.n_tiles, d.sub, s_red);
    V2 = final_sum(d.part + d.n_units, d.n_tiles, d.sub, s_red);
    F2 = final_sum(d.part + 2 * (size_t)d.n_units, d.n_tiles, d.sub, s_red);
    M2 = final_max(d.part + 3 * (size_t)d.n_units, d.n_units, s_red);
}

/* ------------------------------------------------------------------ */

/* kGel: the network carries a gel (network_mesh_relax.cu); the instance
 * without it has no gel code. */
/* stall > 0 makes every grid barrier wait for that many CTAs that do not
 * exist, so the first wait runs out of its budget: the failure-detection
 * test of the wait budget (NR_TEST_STALL_BARRIER). */
template <bool kGel>
__global__ void k_fire_grid(NetDev d, FireParamsDev p, unsigned long long budget_ns, unsigned stall) {
    extern __shared__ double s_units[];
    __shared__ double s_red[32]; /* one slot per warp, up to 1024 threads */
    const unsigned G = gridDim.x, GB = G + stall;
    Scal s;
    bool last;
    const int item0 = blockIdx.x * blockDim.x + threadIdx.x, istride = G * blockDim.x;
    items_pass<kGel>(d, item0, istride);
    if (!barrier_arrive(d.st, GB, budget_ns, last, 4)) return;
    if (last) barrier_release(d.st);
    pass_b<kGel>(d, 0.0, true, blockIdx.x, G, s_units);
    if (!barrier_arrive(d.st, GB, budget_ns, last, 1)) return;
    if (last) {
        double P, V2, F2, M2;
        reduce_parts(d, s_red, P, V2, F2, M2);
        if (threadIdx.x == 0) { /* FP64 scalars: one thread (GB300 FP64 is scarce) */
            scal_init(s, p, F2, M2, d.sqrt_dof);
            scal_store(d.st, s);
        }
        barrier_release(d.st);
    }
    for (;;) {
        scal_load(s, d.st);
        pass_a(d, s, blockIdx.x, G);
        if (s.done) break;
        if (!barrier_arrive(d.st, GB, budget_ns, last, 2)) return;
        if (last) barrier_release(d.st);
        items_pass<kGel>(d, item0, istride);
        if (!barrier_arrive(d.st, GB, budget_ns, last, 5)) return;
        if (last) barrier_release(d.st);
        pass_b<kGel>(d, s.dtm, false, blockIdx.x, G, s_units);
        if (!barrier_arrive(d.st, GB, budget_ns, last, 3)) return;
        if (last) {
            double P, V2, F2, M2;
            reduce_parts(d, s_red, P, V2, F2, M2);
            if (threadIdx.x == 0) {
                scal_step(s, p, P, V2, F2, M2, d.sqrt_dof);
                scal_store(d.st, s);
            }
            barrier_release(d.st);
        }
    }
}

__global__ void k_energy_tiles(NetDev d) {
    __shared__ double s_red[32]; /* one slot per warp, up to 1024 threads */
    energy_tiles(d, blockIdx.x, gridDim.x, s_red);
}

__global__ void k_energy_final(NetDev d) {
    __shared__ double s_red[32]; /* one slot per warp, up to 1024 threads */
    double es, eb, eg, vir[3];
    energy_final(d, s_red, es, eb, eg, vir);
    if (threadIdx.x == 0) {
        d.st->e_stretch = es;
        d.st->e_bend = eb;
        d.st->e_gel = eg;
        for (int c = 0; c < 3; ++c) d.st->vir[c] = vir[c];
    }
}

/* One CTA per network, networks taken from *queue until exhausted
 * (batches carry no gel). */
__global__ void __launch_bounds__(256) k_fire_batch(const NetDev *nets, int n_nets, FireParamsDev p, int *queue) {
    extern __shared__ double s_units[];
    __shared__ double s_red[32]; /* one slot per warp, up to 1024 threads */
    __shared__ int s_net;
    __shared__ NetDev s_d; /* descriptor staged once per network (hoistable loads) */
    __shared__ Scal s_sc;  /* FIRE scalars, advanced by thread 0 (GB300 FP64 is scarce) */
    for (;;) {
        if (threadIdx.x == 0) {
            s_net = atomicAdd(queue, 1);
            if (s_net < n_nets) s_d = nets[s_net];
        }
        __syncthreads();
        const int net = s_net;
        if (net >= n_nets) return;
        const NetDev &d = s_d;
        double P, V2, F2, M2;
        items_pass<false>(d, threadIdx.x, blockDim.x);
        __syncthreads();
        pass_b<false>(d, 0.0, true, 0, 1, s_units);
        reduce_parts(d, s_red, P, V2, F2, M2);
        if (threadIdx.x == 0) scal_init(s_sc, p, F2, M2, d.sqrt_dof);
        __syncthreads();
        for (;;) {
            pass_a(d, s_sc, 0, 1);
            if (s_sc.done) break;
            __syncthreads();
            items_pass<false>(d, threadIdx.x, blockDim.x);
            __syncthreads();
            pass_b<false>(d, s_sc.dtm, false, 0, 1, s_units);
            reduce_parts(d, s_red, P, V2, F2, M2);
            if (threadIdx.x == 0) scal_step(s_sc, p, P, V2, F2, M2, d.sqrt_dof);
            __syncthreads();
        }
        __syncthreads();
        energy_tiles<false>(d, 0, 1, s_red);
        double es, eb, eg, vir[3];
        energy_final(d, s_red, es, eb, eg, vir);
        if (threadIdx.x == 0) {
            scal_store(d.st, s_sc);
            d.st->e_stretch = es;
            d.st->e_bend = eb;
            d.st->e_gel = eg;
            for (int c = 0; c < 3; ++c) d.st->vir[c] = vir[c];
        }
        __syncthreads();
    }
}

/* ------------------------------------------------------------------ */
/* One thread-block cluster per network (FP64)                          */
/* ------------------------------------------------------------------ */

/* The FP64 step of k_fire_grid with the software grid barrier replaced by
 * the hardware cluster barrier: a network is relaxed by the C CTAs (C SMs,
 * up to 16) of one cluster.  Every warp of the cluster takes 32-node chunks
 * (unit = one chunk: the canonical reduction with sub = 1), items are spread
 * over all the cluster's threads, and after the barrier that ends pass B
 * EVERY CTA reduces the unit partials itself, in the canonical order, so
 * every CTA's thread 0 advances an identical copy of the FIRE scalars and no
 * fourth barrier is needed.  Same operations on the same values as
 * k_fire_grid and the oracle: the same bits.  On small networks the grid
 * kernel's step is set by the latency of its three software barriers (about
 * 40 us); these barriers are hardware ones.  Persistent over a work queue:
 * one network (nr_relax) or a batch (nr_batch_relax). */
template <bool kGel>
__global__ void __launch_bounds__(kTile, 1)
    k_fire_cluster(const NetDev *nets, int n_nets, FireParamsDev p, int *queue, const int *order) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    __shared__ double s_red[32];
    __shared__ NetDev s_d;
    __shared__ Scal s_sc;
    __shared__ int s_slot;
    const int rank = (int)cl.block_rank(), C = (int)cl.num_blocks();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wpc = blockDim.x >> 5;
    const int gw = rank * wpc + warp, nw = C * wpc; /* warps of the cluster */
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) s_slot = atomicAdd(queue, 1);
        cl.sync();
        const int slot = *cl.map_shared_rank(&s_slot, 0);
        /* every CTA has read rank 0's slot before any CTA may exit or rank 0
         * overwrites it for the next network */
        cl.sync();
        if (slot >= n_nets) return;
        if (threadIdx.x == 0) s_d = nets[order ? order[slot] : slot];
        __syncthreads();
        const NetDev &d = s_d;
        const int n_units = d.n_tiles * 8; /* 32-node chunks, padded to whole tiles */
        const int item0 = rank * blockDim.x + threadIdx.x, istride = C * blockDim.x;
        bool init = true;
        for (;;) {
            if (!init) {
                for (int u = gw; u * kChunk < d.n; u += nw) {
                    const int i = u * kChunk + lane;
                    if (i < d.n) pass_a_node(d, s_sc, i);
                }
                if (s_sc.done) break;
                cl.sync();
            }
            items_pass<kGel>(d, item0, istride);
            cl.sync();
            /* pass B: gather, half kick (v = 0 at the start), unit partials */
            const double dtm = init ? 0.0 : s_sc.dtm;
            for (int u = gw; u < n_units; u += nw) {
                const int i = u * kChunk + lane;
                double tP = 0.0, tV = 0.0, tF = 0.0;
                if (i < d.n) {
                    double fx, fy;
                    node_force_items<kGel>(d, i, fx, fy);
                    double2 vi;
                    if (init) {
                        vi = make_double2(0.0, 0.0);
                    } else {
                        vi = d.v[i];
                        vi.x = fma(dtm, fx, vi.x);
                        vi.y = fma(dtm, fy, vi.y);
                    }
                    d.v[i] = vi;
                    d.f[i] = make_double2(fx, fy);
                    tP = dot2(vi.x, vi.y, fx, fy);
                    tV = dot2(vi.x, vi.y, vi.x, vi.y);
                    tF = dot2(fx, fy, fx, fy);
                }
                const double sP = warp_sum(tP), sV = warp_sum(tV), sF = warp_sum(tF), sM = warp_max(tF);
                if (lane == 0) {
                    d.part[u] = sP;
                    d.part[(size_t)n_units + u] = sV;
                    d.part[2 * (size_t)n_units + u] = sF;
                    d.part[3 * (size_t)n_units + u] = sM;
                }
            }
            cl.sync();
            /* every CTA: the canonical totals and the FIRE scalars */
            const double P = final_sum(d.part, d.n_tiles, 1, s_red);
            const double V2 = final_sum(d.part + n_units, d.n_tiles, 1, s_red);
            const double F2 = final_sum(d.part + 2 * (size_t)n_units, d.n_tiles, 1, s_red);
            const double M2 = final_max(d.part + 3 * (size_t)n_units, n_units, s_red);
            if (threadIdx.x == 0) {
                if (init) scal_init(s_sc, p, F2, M2, d.sqrt_dof);
                else scal_step(s_sc, p, P, V2, F2, M2, d.sqrt_dof);
            }
            __syncthreads();
            init = false;
        }
        cl.sync();
        energy_tiles<kGel>(d, rank, C, s_red);
        cl.sync();
        if (rank == 0) {
            double es, eb, eg, vir[3];
            energy_final(d, s_red, es, eb, eg, vir);
            if (threadIdx.x == 0) {
                scal_store(d.st, s_sc);
                d.st->e_stretch = es;
                d.st->e_bend = eb;
                d.st->e_gel = eg;
                for (int c = 0; c < 3; ++c) d.st->vir[c] = vir[c];
            }
        }
        cl.sync();
    }
}

__global__ void k_forces(NetDev d) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n) return;
    double fx, fy;
    node_force_fp64(d, i, fx, fy);
    d.f[i] = make_double2(fx, fy);
}

/* affine_displace (large_strain_relax.cu:527-537) over N nodes; with
 * --fmad=false the operations round exactly as the reference's. */
__global__ void k_affine(double2 *x, int n, double miny, double yrange, double xdisp, double ydisp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 p = x[i];
    const double dy = p.y - miny;
    p.x = p.x + xdisp * dy / yrange;
    p.y = p.y + ydisp * dy / yrange;
    x[i] = p;
}

/* get_inv_mats (network_mesh_relax.cu:503-531): the inverse of each gel
 * triangle's reference matrix from positions pos (2N doubles); vertex v of
 * element e is facets[stride * e + v] (stride 3: the reference's list, 4:
 * int4 records).  Plain IEEE operations in the reference's order
 * (--fmad=false), as the oracle computes them. */
__global__ void k_inv_mats(const double *pos, const int *facets, int stride, int n_elems, double *inv) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n_elems) return;
    const int i1 = facets[(size_t)stride * e], i2 = facets[(size_t)stride * e + 1], i3 = facets[(size_t)stride * e + 2];
    const double x1 = pos[2 * (size_t)i1], y1 = pos[2 * (size_t)i1 + 1];
    const double x2 = pos[2 * (size_t)i2], y2 = pos[2 * (size_t)i2 + 1];
    const double x3 = pos[2 * (size_t)i3], y3 = pos[2 * (size_t)i3 + 1];
    const double det = x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2);
    double *M = inv + 6 * (size_t)e;
    M[0] = (y2 - y3) / det;
    M[1] = (x3 - x2) / det;
    M[2] = (y3 - y1) / det;
    M[3] = (x1 - x3) / det;
    M[4] = (y1 - y2) / det;
    M[5] = (x2 - x1) / det;
}

/* dilate (network_mesh_relax.cu:796-806) over N nodes. */
__global__ void k_dilate(double2 *x, int n, double minx, double miny, double factor) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double2 p = x[i];
    p.x = minx + factor * (p.x - minx);
    p.y = miny + factor * (p.y - miny);
    x[i] = p;
}

/* Per-network affine map for a batch: one CTA per network. */
__global__ void k_affine_batch(const NetDev *nets, const double4 *prm) {
    const NetDev d = nets[blockIdx.x];
    const double4 q = prm[blockIdx.x]; /* miny, yrange, xdisp, ydisp */
    for (int i = threadIdx.x; i < d.n; i += blockDim.x) {
        double2 p = d.x[i];
        const double dy = p.y - q.x;
        p.x = p.x + q.z * dy / q.y;
        p.y = p.y + q.w * dy / q.y;
        d.x[i] = p;
    }
}

/* ------------------------------------------------------------------ */
/* Host launchers                                                       */
/* ------------------------------------------------------------------ */

static size_t grid_smem_bytes(int sub) { return (size_t)kGroup * 4 * sub * sizeof(double); }

cudaError_t fp64_grid_max_blocks(int sub, bool gel, int *max_blocks) {
    int dev, sms, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gel ? k_fire_grid<true> : k_fire_grid<false>, 32 * sub,
                                                      grid_smem_bytes(sub));
    if (e != cudaSuccess) return e;
    *max_blocks = per_sm * sms;
    return cudaSuccess;
}

cudaError_t launch_fp64_grid(const NetDev &d, const FireParamsDev &p, int blocks, unsigned long long budget_ns,
                             unsigned stall, cudaStream_t stream) {
    NetDev dd = d;
    FireParamsDev pp = p;
    unsigned long long bb = budget_ns;
    unsigned ss = stall;
    void *args[] = {&dd, &pp, &bb, &ss};
    const void *k = d.use_gel ? (const void *)k_fire_grid<true> : (const void *)k_fire_grid<false>;
    return launch_cooperative(k, blocks, 32 * d.sub, args, grid_smem_bytes(d.sub), stream);
}

cudaError_t launch_energies(const NetDev &d, int blocks, cudaStream_t stream) {
    k_energy_tiles<<<blocks, kTile, 0, stream>>>(d);
    k_energy_final<<<1, kTile, 0, stream>>>(d);
    return cudaGetLastError();
}

cudaError_t launch_fp64_batch(const NetDev *nets_dev, int n_nets, const FireParamsDev &p, int *queue_dev,
                              int blocks, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(queue_dev, 0, sizeof(int), stream);
    if (e != cudaSuccess) return e;
    k_fire_batch<<<blocks, kTile, grid_smem_bytes(8), stream>>>(nets_dev, n_nets, p, queue_dev);
    return cudaGetLastError();
}

cudaError_t fp64_batch_max_blocks(int *max_blocks) {
    int dev, sms, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fire_batch, kTile, grid_smem_bytes(8));
    if (e != cudaSuccess) return e;
    *max_blocks = per_sm * sms;
    return cudaSuccess;
}

/* Clusters of C CTAs that fit the GPU at once (0: the size cannot run). */
cudaError_t fp64_cluster_max_active(int cluster, bool gel, int *out) {
    const void *k = gel ? (const void *)k_fire_cluster<true> : (const void *)k_fire_cluster<false>;
    cudaError_t e;
    if (cluster > 8 && (e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) != cudaSuccess)
        return e;
    int dev, sms;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((sms / cluster) * cluster);
    cfg.blockDim = dim3(kTile);
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    *out = 0;
    return cudaOccupancyMaxActiveClusters(out, k, &cfg);
}

cudaError_t launch_fp64_cluster(const NetDev *nets_dev, int n_nets, int cluster, bool gel, const FireParamsDev &p,
                                int *queue_dev, const int *order_dev, cudaStream_t stream) {
    if (cluster < 1 || cluster > 16) return cudaErrorInvalidValue;
    int max_clusters = 0;
    cudaError_t e = fp64_cluster_max_active(cluster, gel, &max_clusters);
    if (e != cudaSuccess) return e;
    if (max_clusters < 1) return cudaErrorLaunchOutOfResources;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(std::max(1, std::min(n_nets, max_clusters)) * cluster);
    cfg.blockDim = dim3(kTile);
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if ((e = cudaMemsetAsync(queue_dev, 0, sizeof(int), stream)) != cudaSuccess) return e;
    if (gel) return cudaLaunchKernelEx(&cfg, k_fire_cluster<true>, nets_dev, n_nets, p, queue_dev, order_dev);
    return cudaLaunchKernelEx(&cfg, k_fire_cluster<false>, nets_dev, n_nets, p, queue_dev, order_dev);
}

cudaError_t launch_forces(const NetDev &d, cudaStream_t stream) {
    k_forces<<<(d.n + 255) / 256, 256, 0, stream>>>(d);
    return cudaGetLastError();
}

cudaError_t launch_affine(double2 *x, int n, double miny, double yrange, double xdisp, double ydisp,
                          cudaStream_t stream) {
    k_affine<<<(n + 255) / 256, 256, 0, stream>>>(x, n, miny, yrange, xdisp, ydisp);
    return cudaGetLastError();
}

cudaError_t launch_inv_mats(const double *pos, const int *facets, int stride, int n_elems, double *inv,
                            cudaStream_t stream) {
    if (n_elems <= 0) return cudaSuccess;
    k_inv_mats<<<(n_elems + 255) / 256, 256, 0, stream>>>(pos, facets, stride, n_elems, inv);
    return cudaGetLastError();
}

cudaError_t launch_dilate(double2 *x, int n, double minx, double miny, double factor, cudaStream_t stream) {
    k_dilate<<<(n + 255) / 256, 256, 0, stream>>>(x, n, minx, miny, factor);
    return cudaGetLastError();
}

cudaError_t launch_affine_batch(const NetDev *nets_dev, const double4 *prm_dev, int n_nets, cudaStream_t stream) {
    k_affine_batch<<<n_nets, 256, 0, stream>>>(nets_dev, prm_dev);
    return cudaGetLastError();
}

}  // namespace nr
