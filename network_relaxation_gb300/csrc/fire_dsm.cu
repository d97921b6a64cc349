/*
 * Mixed-precision FIRE with the per-step state in distributed shared memory.
 *
 * One thread-block cluster of C CTAs relaxes one network at a time (a
 * persistent kernel over the batch's work queue).  Every value a FIRE step
 * writes and reads back lives in the cluster's shared memory:
 *   per node (owner CTA)   u (double-float, float4), FP32 v, FP32 F
 *   per item (owner CTA)   the FP32 force change of the current step
 * A CTA reads another CTA's u (item pass) or item results (gather) with
 * ld.shared::cluster on addresses from mapa, after the hardware cluster
 * barrier that ends the producing pass.  Only read-only data comes from
 * global memory during a step: topology (read-only cache), the anchor
 * records and the anchor force (rewritten only at anchors, by the CTA that
 * reads them).  In the global-memory cluster kernel (fire_mixed.cu) each
 * pass paid dependent L2 round trips; here a step costs three cluster
 * barriers and on-chip latencies.
 *
 * The arithmetic (bond_dforce, tri_dforce, double-float u, the FP32 FIRE
 * step and the FP64 anchors and certification) is mixed_common.cuh's,
 * unchanged.  Layout: NetDsm (nr_device.cuh).  Shared memory per CTA:
 * 32 B per owned node + 8 B per owned bond + 16 B per owned triple; the
 * host uses this kernel when the largest network of the batch fits.
 *
 * Compiled with --fmad=false; FP32 expressions use explicit fmaf().
 */
#include "mixed_common.cuh"

namespace nr {

/* 32-bit shared::cluster address of shared-memory location p in CTA `rank`. */
__device__ __forceinline__ unsigned dsm_addr(const void *p, unsigned rank) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ float2 dsm_ld2(unsigned a) {
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
    return v;
}
__device__ __forceinline__ float4 dsm_ld4(unsigned a) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(a));
    return v;
}

/* Shared::cluster address of the u of node reference `ref` (sub-block << 16
 * | index in it) when each CTA owns spr = 2^lg sub-blocks of bsub nodes;
 * au[r] = address of CTA r's s_u. */
__device__ __forceinline__ unsigned u_addr(const unsigned *au, int ref, int lg, int bsub) {
    const int sb = (int)((unsigned)ref >> 16), r = sb >> lg;
    const int local = (sb & ((1 << lg) - 1)) * bsub + (ref & 0xffff);
    return au[r] + 16u * (unsigned)local;
}

/* Anchor step 2 for the CTA's own items and nodes: FP32 anchor records by
 * slot, FP64 forces into f, the double-float anchor force, F = F(X) in
 * shared memory; CTA partials of |F|^2 and max|F|^2 in F2, M2. */
static __device__ __noinline__ void anchor_eval_dsm(const NetDev &d, const NetDsm &m, int n0, int nloc, int b0, int b1,
                                                    int t0, int t1, float2 *s_f, double &F2, double &M2) {
    const double W = d.width;
    F2 = 0.0;
    M2 = 0.0;
    if (d.use_bonds)
        for (int sl = b0 + threadIdx.x; sl < b1; sl += blockDim.x) {
            const int b = __ldg(m.bidx + sl);
            const int4 r = __ldg(d.bond + b);
            const double2 p1 = d.x[r.x], p2 = d.x[r.y];
            const double rx = (p2.x + wrap_shift(r.z, W)) - p1.x, ry = p2.y - p1.y;
            const double k = d.bond_k ? d.bond_k[b] : d.ks;
            const float hx = (float)rx, hy = (float)ry;
            d.mb_data[sl] = make_float4(hx, hy, (float)(rx - (double)hx), (float)(ry - (double)hy));
            d.mb_sk[sl] = make_float2((float)(sqrt(fma(rx, rx, ry * ry)) - d.bond_l0[b]), (float)k);
        }
    if (d.use_triples)
        for (int sl = t0 + threadIdx.x; sl < t1; sl += blockDim.x) {
            const int t = __ldg(m.tref + sl).w;
            const int4 r = __ldg(d.tri + t);
            const double2 ph = d.x[r.x], pj = d.x[r.y], pk = d.x[r.z];
            const int wj = (signed char)(r.w & 0xff), wk = (signed char)((r.w >> 8) & 0xff);
            const double ax = (pj.x + wrap_shift(wj, W)) - ph.x, ay = pj.y - ph.y;
            const double bx = (pk.x + wrap_shift(wk, W)) - ph.x, by = pk.y - ph.y;
            const double kb = d.tri_kb ? d.tri_kb[t] : d.kb;
            const double phi0 = d.tri_phi0 ? d.tri_phi0[t] : 0.0;
            d.mt_arms[sl] = make_float4((float)ax, (float)ay, (float)bx, (float)by);
            d.mt_pk[sl] = make_float2((float)bend_dtheta(ax, ay, bx, by, phi0), (float)kb);
        }
    for (int li = threadIdx.x; li < nloc; li += blockDim.x) {
        const int i = n0 + li;
        double fx, fy;
        node_force_fp64(d, i, fx, fy);
        d.f[i] = make_double2(fx, fy);
        const float hx = (float)fx, hy = (float)fy;
        d.fa_hi[i] = make_float2(hx, hy);
        d.fa_lo[i] = make_float2((float)(fx - (double)hx), (float)(fy - (double)hy));
        s_f[li] = make_float2(hx, hy);
        const double t = dot2(fx, fy, fx, fy);
        F2 += t;
        M2 = fmax(M2, t);
    }
}

template <int NT>
__global__ void __launch_bounds__(NT, 1)
    k_fire_dsm_mixed(const NetDev *nets, const NetDsm *dsms, int n_nets, FireParamsDev p, int *queue,
                     const int *order, int bmax, int emax, int tmax, int yield_at) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ float4 s_dyn[];
    float4 *s_u = s_dyn;                       /* [bmax] {hi.x, hi.y, lo.x, lo.y} */
    float4 *s_tdf = s_u + bmax;                /* [tmax] */
    float2 *s_v = reinterpret_cast<float2 *>(s_tdf + tmax); /* [bmax] */
    float2 *s_f = s_v + bmax;                  /* [bmax] */
    float2 *s_bdf = s_f + bmax;                /* [emax] */
    __shared__ MixShared sh;
    __shared__ NetDev s_d;
    __shared__ NetDsm s_m;
    __shared__ int s_slot;
    __shared__ Part s_part;
    __shared__ double s_anc[2];
    __shared__ int s_yield; /* rank 0: half the clusters are idle, escalate */
    __shared__ int s_flag;  /* network start: resume a yielded network; in the loop: leave after this anchor */
    __shared__ unsigned s_au[kDsmParts], s_ab[kDsmParts], s_at[kDsmParts];
    const int rank = (int)cl.block_rank(), C = (int)cl.num_blocks();
    const int spr = kDsmParts / C, lg = __ffs(spr) - 1; /* sub-blocks per CTA, log2 */
    if ((int)threadIdx.x < C) {
        s_au[threadIdx.x] = dsm_addr(s_u, threadIdx.x);
        s_ab[threadIdx.x] = dsm_addr(s_bdf, threadIdx.x);
        s_at[threadIdx.x] = dsm_addr(s_tdf, threadIdx.x);
    }
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) s_slot = atomicAdd(queue, 1);
        cl.sync();
        const int slot = *cl.map_shared_rank(&s_slot, 0);
        /* every CTA has read rank 0's slot before any CTA may exit (a CTA's
         * shared memory must not be read remotely after it exits) or rank 0
         * overwrites it for the next network */
        cl.sync();
        if (slot >= n_nets) {
            if (rank == 0 && threadIdx.x == 0) atomicAdd(queue + 1, 1); /* one more idle cluster */
            return;
        }
        if (threadIdx.x == 0) {
            const int idx = order ? order[slot] : slot;
            s_d = nets[idx];
            s_m = dsms[idx];
        }
        __syncthreads();
        const NetDev &d = s_d;
        const NetDsm &m = s_m;
        const int bsub = m.bsub;
        const int n0 = rank * spr * bsub, nloc = max(0, min(spr * bsub, d.n - n0));
        const int b0 = m.bo[rank * spr], b1 = m.bo[(rank + 1) * spr];
        const int t0 = m.to[rank * spr], t1 = m.to[(rank + 1) * spr];
        if (threadIdx.x == 0) s_flag = ((volatile FireState *)d.st)->yielded;
        __syncthreads();
        MixScal s; /* replicated in thread 0 of every CTA */
        MixParams q;
        double F2, M2, tF2, tM2;
        if (s_flag) {
            /* resume a network a smaller cluster left at an anchor: u = 0,
             * v and the FIRE scalars saved, F = F(X) and the anchor records
             * in global memory (slot-indexed: the layout does not depend on
             * the cluster size) */
            for (int li = threadIdx.x; li < nloc; li += NT) {
                s_u[li] = make_float4(0.f, 0.f, 0.f, 0.f);
                s_v[li] = d.vf[n0 + li];
                s_f[li] = d.fa_hi[n0 + li];
            }
            if (threadIdx.x == 0) {
                s = mix_load(d.st);
                q = mix_params(p, d.sqrt_dof);
                sh.coef = coef_of(s, 0);
            }
            __syncthreads();
        } else {
            for (int li = threadIdx.x; li < nloc; li += NT) {
                s_u[li] = make_float4(0.f, 0.f, 0.f, 0.f);
                s_v[li] = make_float2(0.f, 0.f);
            }
            anchor_eval_dsm(d, m, n0, nloc, b0, b1, t0, t1, s_f, F2, M2);
            anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
            if (threadIdx.x == 0) {
                s_anc[0] = tF2;
                s_anc[1] = tM2;
            }
            cl.sync();
            if (threadIdx.x == 0) {
                double t[2];
                anchor_totals(cl, s_anc, t);
                q = mix_params(p, d.sqrt_dof);
                mix_init(s, q);
                mix_certify(s, p, d.sqrt_dof, t[0], t[1]);
                sh.coef = coef_of(s, 0);
            }
            __syncthreads();
        }
        for (;;) {
            const Coef c = sh.coef;
            /* pass A: mixing, drift, half kick of the owned nodes */
            for (int li = threadIdx.x; li < nloc; li += NT) {
                float2 v = s_v[li];
                const float2 F = s_f[li];
                if (c.mix_pending) {
                    v.x = fmaf(c.na, v.x, v.x);
                    v.y = fmaf(c.na, v.y, v.y);
                    v.x = fmaf(c.a, F.x, v.x);
                    v.y = fmaf(c.a, F.y, v.y);
                    if (c.zero_v) v = make_float2(0.f, 0.f);
                }
                if (!c.done) {
                    float4 u = s_u[li];
                    df_add(u.x, u.z, fmaf(c.dt, v.x, c.dtsq * F.x));
                    df_add(u.y, u.w, fmaf(c.dt, v.y, c.dtsq * F.y));
                    s_u[li] = u;
                    v.x = fmaf(c.dtm, F.x, v.x);
                    v.y = fmaf(c.dtm, F.y, v.y);
                }
                s_v[li] = v;
            }
            if (c.done) break;
            cl.sync();
            /* item pass: owned bonds and triples, u of any CTA.  Software
             * pipelined: the next item's reference and anchor record (read
             * only, mostly from L2) are loaded while the current one computes */
            if (d.use_bonds) {
                int sl = b0 + threadIdx.x;
                if (sl < b1) {
                    int2 r = __ldg(m.bref + sl);
                    float4 ra = d.mb_data[sl];
                    float2 sk = d.mb_sk[sl];
                    for (;;) {
                        const float4 ui = dsm_ld4(u_addr(s_au, r.x, lg, bsub));
                        const float4 uj = dsm_ld4(u_addr(s_au, r.y, lg, bsub));
                        const int nx = sl + NT;
                        int2 rn = r;
                        float4 ran = ra;
                        float2 skn = sk;
                        if (nx < b1) {
                            rn = __ldg(m.bref + nx);
                            ran = d.mb_data[nx];
                            skn = d.mb_sk[nx];
                        }
                        float2 dh, dlo;
                        u_diff2(make_float2(uj.x, uj.y), make_float2(uj.z, uj.w), make_float2(ui.x, ui.y),
                                make_float2(ui.z, ui.w), dh, dlo);
                        s_bdf[sl - b0] = bond_dforce(ra, sk, dh, dlo);
                        if (nx >= b1) break;
                        sl = nx;
                        r = rn;
                        ra = ran;
                        sk = skn;
                    }
                }
            }
            if (d.use_triples) {
                int sl = t0 + threadIdx.x;
                if (sl < t1) {
                    int4 r = __ldg(m.tref + sl);
                    float4 arms = d.mt_arms[sl];
                    float2 pk = d.mt_pk[sl];
                    for (;;) {
                        const float4 uh = dsm_ld4(u_addr(s_au, r.x, lg, bsub));
                        const float4 uj = dsm_ld4(u_addr(s_au, r.y, lg, bsub));
                        const float4 uk = dsm_ld4(u_addr(s_au, r.z, lg, bsub));
                        const int nx = sl + NT;
                        int4 rn = r;
                        float4 armsn = arms;
                        float2 pkn = pk;
                        if (nx < t1) {
                            rn = __ldg(m.tref + nx);
                            armsn = d.mt_arms[nx];
                            pkn = d.mt_pk[nx];
                        }
                        const float2 hh = make_float2(uh.x, uh.y), hl = make_float2(uh.z, uh.w);
                        float2 dFj, dFk;
                        tri_dforce(arms, pk, u_diff(make_float2(uj.x, uj.y), make_float2(uj.z, uj.w), hh, hl),
                                   u_diff(make_float2(uk.x, uk.y), make_float2(uk.z, uk.w), hh, hl), dFj, dFk);
                        s_tdf[sl - t0] = make_float4(dFj.x, dFj.y, dFk.x, dFk.y);
                        if (nx >= t1) break;
                        sl = nx;
                        r = rn;
                        arms = armsn;
                        pk = pkn;
                    }
                }
            }
            cl.sync();
            /* gather: F = F(X) + the node's entries in incidence order, half kick */
            float P = 0.f, V2 = 0.f, Fs = 0.f, M2f = 0.f, A = 0.f;
            for (int li = threadIdx.x; li < nloc; li += NT) {
                const int i = n0 + li;
                /* the node's independent global loads first: one round trip */
                const unsigned fc = __ldg(d.fcode + i);
                const int be0 = __ldg(d.bptr + i), be1 = __ldg(d.bptr + i + 1);
                const int te0 = __ldg(d.tptr + i), te1 = __ldg(d.tptr + i + 1);
                const float2 ah = d.fa_hi[i], al = d.fa_lo[i];
                float2 F = make_float2(0.f, 0.f);
                if (fc != 0) {
                    float2 dF = make_float2(0.f, 0.f);
                    float mag = 0.f;
                    if (d.use_bonds) {
#pragma unroll 4
                        for (int e = be0; e < be1; ++e) {
                            const unsigned code = (unsigned)__ldg(m.bent + e);
                            const int r = (int)(code >> 28) >> lg;
                            const int ls = (int)((code >> 1) & 0x7ffffffu) - s_m.bo[r * spr];
                            float2 df = dsm_ld2(s_ab[r] + 8u * (unsigned)ls);
                            if (code & 1) df = make_float2(-df.x, -df.y);
                            dF.x += df.x;
                            dF.y += df.y;
                            mag += fabsf(df.x) + fabsf(df.y);
                        }
                    }
                    if (d.use_triples) {
#pragma unroll 4
                        for (int e = te0; e < te1; ++e) {
                            const unsigned code = (unsigned)__ldg(m.tent + e);
                            const int r = (int)(code >> 28) >> lg;
                            const int role = code & 3;
                            const int ls = (int)((code >> 2) & 0x3ffffffu) - s_m.to[r * spr];
                            const float4 qv = dsm_ld4(s_at[r] + 16u * (unsigned)ls);
                            float gx, gy, mg;
                            if (role == 0) {
                                gx = -(qv.x + qv.z);
                                gy = -(qv.y + qv.w);
                                mg = fabsf(qv.x) + fabsf(qv.y) + fabsf(qv.z) + fabsf(qv.w);
                            } else {
                                gx = role == 1 ? qv.x : qv.z;
                                gy = role == 1 ? qv.y : qv.w;
                                mg = fabsf(gx) + fabsf(gy);
                            }
                            dF.x += gx;
                            dF.y += gy;
                            mag += mg;
                        }
                    }
                    A = fmaxf(A, mag);
                    F.x = ah.x + (al.x + dF.x);
                    F.y = ah.y + (al.y + dF.y);
                    if (!(fc & 1)) F.x = 0.f;
                    if (!(fc & 2)) F.y = 0.f;
                }
                float2 v = s_v[li];
                v.x = fmaf(c.dtm, F.x, v.x);
                v.y = fmaf(c.dtm, F.y, v.y);
                s_v[li] = v;
                s_f[li] = F;
                P += fmaf(v.x, F.x, v.y * F.y);
                V2 += fmaf(v.x, v.x, v.y * v.y);
                const float f2 = fmaf(F.x, F.x, F.y * F.y);
                Fs += f2;
                M2f = fmaxf(M2f, f2);
            }
            warp_part(Part{P, V2, Fs, M2f, A}, sh.slots);
            __syncthreads();
            if (threadIdx.x < 32) {
                const Part t = block_totals(sh.slots);
                if (threadIdx.x == 0) {
                    s_part = t;
                    if (rank == 0) s_yield = yield_at > 0 && *(volatile int *)(queue + 1) >= yield_at;
                }
            }
            cl.sync();
            if (threadIdx.x < 32) {
                /* lane r takes rank r's totals: the same butterfly in every CTA */
                Part t{0.f, 0.f, 0.f, 0.f, 0.f};
                if ((int)threadIdx.x < C) t = *cl.map_shared_rank(&s_part, (int)threadIdx.x);
                t = warp_reduce(t);
                if (threadIdx.x == 0) {
                    /* rank 0's escalation flag, the same in every CTA */
                    const int y = *cl.map_shared_rank(&s_yield, 0);
                    mix_step(s, q, t);
                    sh.coef = coef_of(s, need_anchor(s, q, t) || y);
                    s_flag = y;
                }
            }
            __syncthreads();
            if (sh.coef.anchor) {
                /* X += u (FP64, global), u = 0, then the FP64 anchor */
                for (int li = threadIdx.x; li < nloc; li += NT) {
                    const int i = n0 + li;
                    const float4 u = s_u[li];
                    double2 x = d.x[i];
                    x.x = x.x + ((double)u.x + (double)u.z);
                    x.y = x.y + ((double)u.y + (double)u.w);
                    d.x[i] = x;
                    s_u[li] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                cl.sync();
                anchor_eval_dsm(d, m, n0, nloc, b0, b1, t0, t1, s_f, F2, M2);
                anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
                if (threadIdx.x == 0) {
                    s_anc[0] = tF2;
                    s_anc[1] = tM2;
                }
                cl.sync();
                if (threadIdx.x == 0) {
                    double t[2];
                    anchor_totals(cl, s_anc, t);
                    mix_certify(s, p, d.sqrt_dof, t[0], t[1]);
                    sh.coef = coef_of(s, 0);
                    s_flag = s_flag && !s.done;
                }
                __syncthreads();
                if (s_flag) break;
            }
        }
        if (s_flag) {
            /* escalate: keep v and the FIRE scalars for the relaunch */
            for (int li = threadIdx.x; li < nloc; li += NT) d.vf[n0 + li] = s_v[li];
            if (rank == 0 && threadIdx.x == 0) {
                d.st->mix = s;
                d.st->yielded = 1;
            }
            continue;
        }
        for (int li = threadIdx.x; li < nloc; li += NT) {
            const float2 v = s_v[li];
            d.v[n0 + li] = make_double2((double)v.x, (double)v.y);
        }
        cl.sync();
        if (rank == 0) {
            mixed_energies(d, sh.red);
            if (threadIdx.x == 0) {
                mix_report(d.st, s);
                d.st->yielded = 0;
            }
        }
        cl.sync();
    }
}

/* Dynamic shared memory of k_fire_dsm_mixed for the given per-CTA maxima. */
size_t dsm_smem_bytes(int bmax, int emax, int tmax) {
    return (size_t)bmax * 16 + (size_t)tmax * 16 + (size_t)bmax * 16 + (size_t)emax * 8;
}

/* Largest dynamic shared memory the kernel may use on this device. */
size_t dsm_smem_limit() {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, (const void *)k_fire_dsm_mixed<1024>) != cudaSuccess) return 0;
    return optin > (int)fa.sharedSizeBytes ? (size_t)(optin - (int)fa.sharedSizeBytes) : 0;
}

template <int NT>
static cudaError_t dsm_config(int cluster, int bmax, int emax, int tmax, cudaLaunchConfig_t &cfg,
                              cudaLaunchAttribute *attr, int *max_clusters) {
    cudaError_t e;
    int dev, sms;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const size_t smem = dsm_smem_bytes(bmax, emax, tmax);
    if ((e = cudaFuncSetAttribute(k_fire_dsm_mixed<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return e;
    if (cluster > 8 &&
        (e = cudaFuncSetAttribute(k_fire_dsm_mixed<NT>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) !=
            cudaSuccess)
        return e;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg = cudaLaunchConfig_t{};
    cfg.blockDim = dim3(NT);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3((sms / cluster) * cluster);
    *max_clusters = 0;
    return cudaOccupancyMaxActiveClusters(max_clusters, (void *)k_fire_dsm_mixed<NT>, &cfg);
}

template <int NT>
static cudaError_t launch_dsm_nt(const NetDev *nets_dev, const NetDsm *dsm_dev, int n_nets, int cluster, int bmax,
                                 int emax, int tmax, double escalate, const FireParamsDev &p, int *queue_dev,
                                 const int *order_dev, cudaStream_t stream) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    int max_clusters = 0;
    cudaError_t e = dsm_config<NT>(cluster, bmax, emax, tmax, cfg, attr, &max_clusters);
    if (e != cudaSuccess) return e;
    if (max_clusters < 1) return cudaErrorLaunchOutOfResources;
    const int clusters = std::max(1, std::min(n_nets, max_clusters));
    cfg.gridDim = dim3(clusters * cluster);
    cfg.stream = stream;
    const int yield_at = escalate > 0 ? std::max(1, (int)(escalate * clusters)) : 0;
    if ((e = cudaMemsetAsync(queue_dev, 0, 2 * sizeof(int), stream)) != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, k_fire_dsm_mixed<NT>, nets_dev, dsm_dev, n_nets, p, queue_dev, order_dev, bmax,
                              emax, tmax, yield_at);
}

static bool dsm_wide() {
    const char *env = getenv("NR_MIX_THREADS");
    return !(env && atoi(env) == 512);
}

cudaError_t launch_mixed_dsm(const NetDev *nets_dev, const NetDsm *dsm_dev, int n_nets, int cluster, int bmax,
                             int emax, int tmax, double escalate, const FireParamsDev &p, int *queue_dev,
                             const int *order_dev, cudaStream_t stream) {
    if (cluster < 1 || cluster > kDsmParts || (kDsmParts % cluster) != 0) return cudaErrorInvalidValue;
    if (dsm_wide())
        return launch_dsm_nt<1024>(nets_dev, dsm_dev, n_nets, cluster, bmax, emax, tmax, escalate, p, queue_dev,
                                   order_dev, stream);
    return launch_dsm_nt<512>(nets_dev, dsm_dev, n_nets, cluster, bmax, emax, tmax, escalate, p, queue_dev,
                              order_dev, stream);
}

cudaError_t dsm_max_clusters(int cluster, int bmax, int emax, int tmax, int *out) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    return dsm_wide() ? dsm_config<1024>(cluster, bmax, emax, tmax, cfg, attr, out)
                      : dsm_config<512>(cluster, bmax, emax, tmax, cfg, attr, out);
}

}  // namespace nr
