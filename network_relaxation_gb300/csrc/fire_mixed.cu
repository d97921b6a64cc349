/*
 * Mixed-precision FIRE kernels with the per-step state in global memory:
 * one CTA per network (u in shared memory when it fits), one thread-block
 * cluster per network, and one network over the whole GPU (cooperative
 * grid).  The arithmetic and the FIRE scalar logic are in mixed_common.cuh.
 *
 * Compiled with --fmad=false (the FP64 anchor code stays canonical); FP32
 * expressions use explicit fmaf().
 */
#include "mixed_common.cuh"
#include "nr_internal.h"

namespace nr {

__device__ void relax_network_cta_mixed(const NetDev &d, const FireParamsDev &p, float4 *s_u, int smem_nodes,
                                        MixShared &sh) {
    const Team tm{0, 1};
    const UView u{d.n <= smem_nodes ? s_u : d.u};
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        u.u[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        d.vf[i] = make_float2(0.f, 0.f);
    }
    MixScal s; /* meaningful in thread 0 only */
    MixParams q;
    double F2, M2, tF2, tM2;
    anchor_eval(d, tm, F2, M2);
    anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
    if (threadIdx.x == 0) {
        q = mix_params(p, d.sqrt_dof);
        mix_init(s, q);
        mix_certify(s, p, d.sqrt_dof, tF2, tM2);
        sh.coef = coef_of(s, 0);
    }
    __syncthreads();
    for (;;) {
        const Coef c = sh.coef;
        mixed_pass_a(d, tm, c, u);
        if (c.done) break;
        __syncthreads();
        mixed_items(d, tm.first(), tm.stride(), u);
        __syncthreads();
        warp_part(mixed_pass_b(d, tm, c.dtm), sh.slots);
        __syncthreads();
        if (threadIdx.x < 32) {
            const Part t = block_totals(sh.slots);
            if (threadIdx.x == 0) {
                mix_step(s, q, t);
                sh.coef = coef_of(s, need_anchor(s, q, t));
            }
        }
        __syncthreads();
        if (sh.coef.anchor) {
            anchor_move(d, tm, u);
            __syncthreads();
            anchor_eval(d, tm, F2, M2);
            anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
            if (threadIdx.x == 0) {
                mix_certify(s, p, d.sqrt_dof, tF2, tM2);
                sh.coef = coef_of(s, 0);
            }
            __syncthreads();
        }
    }
    mixed_finish(d, tm);
    __syncthreads();
    mixed_energies(d, sh.red);
    if (threadIdx.x == 0) mix_report(d.st, s);
    __syncthreads();
}

template <int NT>
__global__ void __launch_bounds__(NT, 1) k_fire_batch_mixed(const NetDev *nets, int n_nets, FireParamsDev p,
                                                            int *queue, const int *order, int smem_nodes) {
    extern __shared__ float4 s_u[];
    __shared__ MixShared sh;
    __shared__ int s_net;
    /* The network's descriptor is staged in shared memory: its pointer
     * fields are then loop-invariant loads the compiler can hoist (a copy
     * in global memory could alias the state arrays being written). */
    __shared__ NetDev s_d;
    for (;;) {
        if (threadIdx.x == 0) {
            const int slot = atomicAdd(queue, 1);
            s_net = slot;
            if (slot < n_nets) s_d = nets[order ? order[slot] : slot];
        }
        __syncthreads();
        const int slot = s_net;
        if (slot >= n_nets) return;
        relax_network_cta_mixed(s_d, p, s_u, smem_nodes, sh);
        __syncthreads();
    }
}

/* ------------------------------------------------------------------ */
/* One thread-block cluster per network (batched, multi-SM teams)       */
/* ------------------------------------------------------------------ */

/* A network relaxed by the C CTAs of one cluster (C SMs): nodes and items
 * are split over the CTAs (interleaved), u lives in global memory
 * (L2-resident), the hardware cluster barrier orders the passes, and each
 * CTA pushes its totals into every other CTA's shared memory (distributed
 * shared memory stores before the barrier).  Thread 0 of every CTA advances an identical copy of the FIRE
 * scalars from the same totals combined in the same order, so no broadcast
 * is needed. */

template <int NT>
__global__ void __launch_bounds__(NT, 1) k_fire_cluster_mixed(const NetDev *nets, int n_nets, FireParamsDev p,
                                                              int *queue, const int *order) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    __shared__ MixShared sh;
    __shared__ NetDev s_d;
    __shared__ int s_slot;
    __shared__ float s_parts[kDsmParts][5];  /* every CTA's step totals (pushed) */
    __shared__ double s_ancs[kDsmParts][2]; /* every CTA's FP64 anchor totals (pushed) */
    const int rank = (int)cl.block_rank(), C = (int)cl.num_blocks();
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) s_slot = atomicAdd(queue, 1);
        cl.sync();
        const int slot = *cl.map_shared_rank(&s_slot, 0);
        /* every CTA has read rank 0's slot before any CTA may exit (a CTA's
         * shared memory must not be read remotely after it exits) or rank 0
         * overwrites it for the next network */
        cl.sync();
        if (slot >= n_nets) return;
        if (threadIdx.x == 0) s_d = nets[order ? order[slot] : slot];
        __syncthreads();
        const NetDev &d = s_d;
        const Team tm{rank, C};
        const UView u{d.u};
        for (int i = tm.first(); i < d.n; i += tm.stride()) {
            u.u[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            d.vf[i] = make_float2(0.f, 0.f);
        }
        MixScal s; /* replicated in thread 0 of every CTA */
        MixParams q;
        double F2, M2, tF2, tM2;
        anchor_eval(d, tm, F2, M2);
        anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
        if (threadIdx.x == 0) anchor_push(s_ancs, rank, C, tF2, tM2);
        cl.sync();
        if (threadIdx.x == 0) {
            double t[2];
            anchor_totals(s_ancs, C, t);
            q = mix_params(p, d.sqrt_dof);
            mix_init(s, q);
            mix_certify(s, p, d.sqrt_dof, t[0], t[1]);
            sh.coef = coef_of(s, 0);
        }
        __syncthreads();
        for (;;) {
            const Coef c = sh.coef;
            mixed_pass_a(d, tm, c, u);
            if (c.done) break;
            cl.sync();
            mixed_items(d, tm.first(), tm.stride(), u);
            cl.sync();
            warp_part(mixed_pass_b(d, tm, c.dtm), sh.slots);
            __syncthreads();
            if (threadIdx.x < 32) {
                const Part t = block_totals(sh.slots);
                /* lane r pushes this CTA's totals into CTA r */
                if ((int)threadIdx.x < C) {
                    const unsigned a = dsm_addr(&s_parts[rank][0], threadIdx.x);
                    dsm_st1(a, t.P);
                    dsm_st1(a + 4u, t.V2);
                    dsm_st1(a + 8u, t.F2);
                    dsm_st1(a + 12u, t.M2);
                    dsm_st1(a + 16u, t.A);
                }
            }
            cl.sync();
            if (threadIdx.x < 32) {
                /* lane r takes rank r's totals: the same butterfly in every CTA */
                Part t{0.f, 0.f, 0.f, 0.f, 0.f};
                if ((int)threadIdx.x < C)
                    t = Part{s_parts[threadIdx.x][0], s_parts[threadIdx.x][1], s_parts[threadIdx.x][2],
                             s_parts[threadIdx.x][3], s_parts[threadIdx.x][4]};
                t = warp_reduce(t);
                if (threadIdx.x == 0) {
                    mix_step(s, q, t);
                    sh.coef = coef_of(s, need_anchor(s, q, t));
                }
            }
            __syncthreads();
            if (sh.coef.anchor) {
                anchor_move(d, tm, u);
                cl.sync();
                anchor_eval(d, tm, F2, M2);
                anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
                if (threadIdx.x == 0) anchor_push(s_ancs, rank, C, tF2, tM2);
                cl.sync();
                if (threadIdx.x == 0) {
                    double t[2];
                    anchor_totals(s_ancs, C, t);
                    mix_certify(s, p, d.sqrt_dof, t[0], t[1]);
                    sh.coef = coef_of(s, 0);
                }
                __syncthreads();
            }
        }
        mixed_finish(d, tm);
        cl.sync();
        if (rank == 0) {
            mixed_energies(d, sh.red);
            if (threadIdx.x == 0) mix_report(d.st, s);
        }
        cl.sync();
    }
}

/* CTAs per network for a batch: enough that the largest network has at
 * most kNodesPerCta nodes per CTA, a power of two up to the portable
 * cluster size 8. */
constexpr int kNodesPerCta = 2304;
int mixed_cluster_size(int max_nodes) {
    int c = 1;
    while (c < 8 && c * kNodesPerCta < max_nodes) c *= 2;
    return c;
}

/* Threads per CTA of the batch and cluster kernels: NR_MIX_THREADS (512 or
 * 1024), default 1024.  A step is a chain of dependent passes, so more
 * warps per SM hide more of its latency: 1024 threads (64 registers, the
 * FP64 anchor code out of line) ran C4-sized networks 1.3-1.6x faster per
 * step than 512. */
static int mixed_threads() {
    const char *env = knob("NR_MIX_THREADS");
    return env && atoi(env) == 512 ? 512 : 1024;
}

template <int NT>
static cudaError_t launch_cluster_nt(const NetDev *nets_dev, int n_nets, int cluster, const FireParamsDev &p,
                                     int *queue_dev, const int *order_dev, cudaStream_t stream) {
    cudaError_t e;
    int dev, sms;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if (cluster > 8 &&
        (e = cudaFuncSetAttribute(k_fire_cluster_mixed<NT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) !=
            cudaSuccess)
        return e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3((sms / cluster) * cluster);
    int max_clusters = 0;
    if ((e = cudaOccupancyMaxActiveClusters(&max_clusters, (void *)k_fire_cluster_mixed<NT>, &cfg)) != cudaSuccess)
        return e;
    if (max_clusters < 1) return cudaErrorLaunchOutOfResources;
    const int clusters = std::max(1, std::min(n_nets, max_clusters));
    cfg.gridDim = dim3(clusters * cluster);
    if ((e = cudaMemsetAsync(queue_dev, 0, sizeof(int), stream)) != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, k_fire_cluster_mixed<NT>, nets_dev, n_nets, p, queue_dev, order_dev);
}

cudaError_t launch_mixed_cluster(const NetDev *nets_dev, int n_nets, int cluster, const FireParamsDev &p,
                                 int *queue_dev, const int *order_dev, cudaStream_t stream) {
    return mixed_threads() == 1024
               ? launch_cluster_nt<1024>(nets_dev, n_nets, cluster, p, queue_dev, order_dev, stream)
               : launch_cluster_nt<512>(nets_dev, n_nets, cluster, p, queue_dev, order_dev, stream);
}

/* Shared memory for u: the largest network of the batch, capped so one CTA
 * fits an SM. */
static int mixed_smem_nodes(int max_nodes) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int budget = optin - 4096; /* static shared memory + margin */
    const int cap = budget > 0 ? budget / 16 : 0;
    return max_nodes < cap ? max_nodes : cap;
}

template <int NT>
static cudaError_t launch_batch_nt(const NetDev *nets_dev, int n_nets, int max_nodes, const FireParamsDev &p,
                                   int *queue_dev, const int *order_dev, cudaStream_t stream) {
    const int smem_nodes = mixed_smem_nodes(max_nodes);
    const size_t smem = (size_t)smem_nodes * 16;
    cudaError_t e =
        cudaFuncSetAttribute(k_fire_batch_mixed<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev, sms, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fire_batch_mixed<NT>, NT, smem)) !=
        cudaSuccess)
        return e;
    const int blocks = std::max(1, std::min(n_nets, std::max(1, per_sm) * sms));
    if ((e = cudaMemsetAsync(queue_dev, 0, sizeof(int), stream)) != cudaSuccess) return e;
    k_fire_batch_mixed<NT><<<blocks, NT, smem, stream>>>(nets_dev, n_nets, p, queue_dev, order_dev, smem_nodes);
    return cudaGetLastError();
}

cudaError_t launch_mixed_batch(const NetDev *nets_dev, int n_nets, int max_nodes, const FireParamsDev &p,
                               int *queue_dev, const int *order_dev, cudaStream_t stream) {
    return mixed_threads() == 1024 ? launch_batch_nt<1024>(nets_dev, n_nets, max_nodes, p, queue_dev, order_dev, stream)
                                   : launch_batch_nt<512>(nets_dev, n_nets, max_nodes, p, queue_dev, order_dev, stream);
}

/* ------------------------------------------------------------------ */
/* One network over the whole GPU (cooperative team of CTAs)            */
/* ------------------------------------------------------------------ */

/* Combines the FP64 CTA partials part[q * G + c] (q < 2: sum, then max) of
 * all G CTAs in CTA order.  Called by one thread of the last-arriving CTA. */
__device__ void anchor_team_totals(const double *part, int G, double *out) {
    double s = 0.0, m = 0.0;
    for (int c = 0; c < G; ++c) {
        s = s + __ldcg(part + c);
        m = fmax(m, __ldcg(part + G + c));
    }
    out[0] = s;
    out[1] = m;
}

/* Step totals of the G CTAs' FP32 totals fpart[q * G + c], by warp 0 of the
 * last-arriving CTA: lane l accumulates CTAs l, l + 32, ... in order, then
 * the butterfly combines the lanes. */
__device__ __forceinline__ Part team_step_totals(const float *fpart, int G) {
    const int lane = threadIdx.x & 31;
    Part t{0.f, 0.f, 0.f, 0.f, 0.f};
    for (int c = lane; c < G; c += 32) {
        t.P += __ldcg(fpart + c);
        t.V2 += __ldcg(fpart + G + c);
        t.F2 += __ldcg(fpart + 2 * G + c);
        t.M2 = fmaxf(t.M2, __ldcg(fpart + 3 * G + c));
        t.A = fmaxf(t.A, __ldcg(fpart + 4 * G + c));
    }
    return warp_reduce(t);
}

template <int NT>
__global__ void __launch_bounds__(NT, 1) k_fire_grid_mixed(NetDev d, FireParamsDev p, unsigned long long budget_ns) {
    __shared__ MixShared sh;
    const Team tm{(int)blockIdx.x, (int)gridDim.x};
    const unsigned G = gridDim.x;
    FireState *st = d.st;
    const UView u{d.u};
    /* d.part: FP64 anchor partials in [0, 2G), FP32 step totals after them */
    float *fpart = reinterpret_cast<float *>(d.part + 2 * (size_t)G);
    bool last;
    MixParams q; /* thread 0 of the last-arriving CTA uses it */
    if (threadIdx.x == 0) q = mix_params(p, d.sqrt_dof);
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        u.u[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        d.vf[i] = make_float2(0.f, 0.f);
    }
    double F2, M2, tF2, tM2;
    anchor_eval(d, tm, F2, M2);
    anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
    if (threadIdx.x == 0) {
        d.part[blockIdx.x] = tF2;
        d.part[G + blockIdx.x] = tM2;
    }
    if (!barrier_arrive(st, G, budget_ns, last, 11)) return;
    if (last) {
        if (threadIdx.x == 0) {
            double t[2];
            anchor_team_totals(d.part, G, t);
            MixScal s;
            mix_init(s, q);
            mix_certify(s, p, d.sqrt_dof, t[0], t[1]);
            st->mix = s;
            st->anchor_now = 0;
        }
        barrier_release(st);
    }
    for (;;) {
        if (threadIdx.x == 0) sh.coef = coef_of(mix_load(st), 0);
        __syncthreads();
        const Coef c = sh.coef;
        mixed_pass_a(d, tm, c, u);
        if (c.done) break;
        if (!barrier_arrive(st, G, budget_ns, last, 12)) return;
        if (last) barrier_release(st);
        mixed_items(d, tm.first(), tm.stride(), u);
        if (!barrier_arrive(st, G, budget_ns, last, 16)) return;
        if (last) barrier_release(st);
        warp_part(mixed_pass_b(d, tm, c.dtm), sh.slots);
        __syncthreads();
        if (threadIdx.x < 32) {
            const Part t = block_totals(sh.slots);
            if (threadIdx.x == 0) {
                fpart[blockIdx.x] = t.P;
                fpart[G + blockIdx.x] = t.V2;
                fpart[2 * G + blockIdx.x] = t.F2;
                fpart[3 * G + blockIdx.x] = t.M2;
                fpart[4 * G + blockIdx.x] = t.A;
            }
        }
        if (!barrier_arrive(st, G, budget_ns, last, 13)) return;
        if (last) {
            if (threadIdx.x < 32) {
                const Part t = team_step_totals(fpart, G);
                if (threadIdx.x == 0) {
                    MixScal s = mix_load(st);
                    mix_step(s, q, t);
                    st->anchor_now = need_anchor(s, q, t);
                    st->mix = s;
                }
            }
            barrier_release(st);
        }
        if (threadIdx.x == 0) {
            const volatile FireState *vs = st;
            sh.coef.anchor = vs->anchor_now;
        }
        __syncthreads();
        if (sh.coef.anchor) {
            anchor_move(d, tm, u);
            if (!barrier_arrive(st, G, budget_ns, last, 14)) return;
            if (last) barrier_release(st);
            anchor_eval(d, tm, F2, M2);
            anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
            if (threadIdx.x == 0) {
                d.part[blockIdx.x] = tF2;
                d.part[G + blockIdx.x] = tM2;
            }
            if (!barrier_arrive(st, G, budget_ns, last, 15)) return;
            if (last) {
                if (threadIdx.x == 0) {
                    double t[2];
                    anchor_team_totals(d.part, G, t);
                    MixScal s = mix_load(st);
                    mix_certify(s, p, d.sqrt_dof, t[0], t[1]);
                    st->mix = s;
                    st->anchor_now = 0;
                }
                barrier_release(st);
            }
        }
    }
    mixed_finish(d, tm);
    if (blockIdx.x == 0 && threadIdx.x == 0) mix_report(st, mix_load(st));
}

/* Threads per CTA of the cooperative grid kernel: NR_MIX_THREADS (512 or
 * 1024), else by size: 1024 above about a thousand nodes per SM (each
 * thread walks long item and node lists; more warps hide more latency:
 * 1M nodes 102 vs 153 us per step), 512 below (grid barriers dominate:
 * 65K nodes 19.6 vs 22.6 us). */
static int grid_threads(int n) {
    const char *env = knob("NR_MIX_THREADS");
    if (env && (atoi(env) == 512 || atoi(env) == 1024)) return atoi(env);
    return n > 152 * 1024 ? 1024 : 512;
}

template <int NT>
static int grid_blocks_nt(int n) {
    int dev, sms, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fire_grid_mixed<NT>, NT, 0) != cudaSuccess) return 0;
    const int want = (n + NT - 1) / NT;
    return std::max(1, std::min(want, per_sm * sms));
}

int mixed_grid_blocks(int n) { return grid_threads(n) == 1024 ? grid_blocks_nt<1024>(n) : grid_blocks_nt<512>(n); }

cudaError_t launch_mixed_grid(const NetDev &d, const FireParamsDev &p, int blocks, unsigned long long budget_ns,
                              cudaStream_t stream) {
    NetDev dd = d;
    FireParamsDev pp = p;
    unsigned long long bb = budget_ns;
    void *args[] = {&dd, &pp, &bb};
    if (grid_threads(d.n) == 1024)
        return launch_cooperative((const void *)k_fire_grid_mixed<1024>, blocks, 1024, args, 0, stream);
    return launch_cooperative((const void *)k_fire_grid_mixed<512>, blocks, 512, args, 0, stream);
}

}  // namespace nr
