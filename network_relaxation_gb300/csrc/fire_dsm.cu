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
#include "nr_internal.h"

namespace nr {

/* Shared::cluster address of the u of node reference `ref` (sub-block << 16
 * | index in it) when each CTA owns spr = 2^lg sub-blocks of bsub nodes;
 * au[r] = address of CTA r's s_u. */
__device__ __forceinline__ unsigned u_addr(const unsigned *au, int ref, int lg, int bsub) {
    const int sb = (int)((unsigned)ref >> 16), r = sb >> lg;
    const int local = (sb & ((1 << lg) - 1)) * bsub + (ref & 0xffff);
    return au[r] + 16u * (unsigned)local;
}

/* Per-CTA dynamic shared memory: the step's state and, when `resident`,
 * copies of the CTA's read-only slices (item references and anchor
 * records, node pointers and incidence entries, anchor force).  Segments
 * of 16-byte elements first, then 8-byte, then 4-byte ones. */
struct DsmSizes {
    int bmax, emax, tmax;   /* nodes, bonds, triples per CTA */
    int ebmax, etmax;       /* bond / triple incidence entries per CTA */
    int resident;
};
struct DsmLayout {
    size_t u, tdf, mb, arms, tref, grec, v, f, bdf, fahi, falo, sk, pk, bref, bent, tent, total;
};
__host__ __device__ inline DsmLayout dsm_layout(const DsmSizes &z) {
    const size_t R = z.resident ? 1 : 0, bm = (size_t)z.bmax, em = (size_t)z.emax, tm = (size_t)z.tmax;
    DsmLayout L;
    size_t o = 0;
    L.u = o;    o += 16 * bm;
    L.tdf = o;  o += 16 * tm;
    L.mb = o;   o += R * 16 * em;
    L.arms = o; o += R * 16 * tm;
    L.tref = o; o += R * 16 * tm;
    L.grec = o; o += R * 16 * bm;
    L.v = o;    o += 8 * bm;
    L.f = o;    o += 8 * bm;
    L.bdf = o;  o += 8 * em;
    L.fahi = o; o += R * 8 * bm;
    L.falo = o; o += R * 8 * bm;
    L.sk = o;   o += R * 8 * em;
    L.pk = o;   o += R * 8 * tm;
    L.bref = o; o += R * 8 * em;
    L.bent = o; o += R * 4 * (size_t)z.ebmax;
    L.tent = o; o += R * 4 * (size_t)z.etmax;
    L.total = o;
    return L;
}

/* Shared-memory copies the anchor writes besides global memory (null when
 * the CTA is not resident). */
struct DsmRes {
    float4 *mb, *arms;
    float2 *sk, *pk, *fahi, *falo;
};

/* Anchor step 2 for the CTA's own items and nodes: FP32 anchor records by
 * slot, FP64 forces into f, the double-float anchor force, F = F(X) in
 * shared memory; CTA partials of |F|^2 and max|F|^2 in F2, M2. */
static __device__ __noinline__ void anchor_eval_dsm(const NetDev &d, const NetDsm &m, int n0, int nloc, int b0, int b1,
                                                    int t0, int t1, float2 *s_f, DsmRes res, double &F2, double &M2) {
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
            const float4 rec = make_float4(hx, hy, (float)(rx - (double)hx), (float)(ry - (double)hy));
            const float2 sk = make_float2((float)(sqrt(fma(rx, rx, ry * ry)) - d.bond_l0[b]), (float)k);
            d.mb_data[sl] = rec;
            d.mb_sk[sl] = sk;
            if (res.mb) {
                res.mb[sl - b0] = rec;
                res.sk[sl - b0] = sk;
            }
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
            const float4 arms = make_float4((float)ax, (float)ay, (float)bx, (float)by);
            const float2 pkv = make_float2((float)bend_dtheta(ax, ay, bx, by, phi0), (float)kb);
            d.mt_arms[sl] = arms;
            d.mt_pk[sl] = pkv;
            if (res.arms) {
                res.arms[sl - t0] = arms;
                res.pk[sl - t0] = pkv;
            }
        }
    for (int li = threadIdx.x; li < nloc; li += blockDim.x) {
        const int i = n0 + li;
        double fx, fy;
        node_force_fp64_own<false>(d, i, fx, fy);
        d.f[i] = make_double2(fx, fy);
        const float hx = (float)fx, hy = (float)fy;
        const float2 fh = make_float2(hx, hy), fl = make_float2((float)(fx - (double)hx), (float)(fy - (double)hy));
        d.fa_hi[i] = fh;
        d.fa_lo[i] = fl;
        if (res.fahi) {
            res.fahi[li] = fh;
            res.falo[li] = fl;
        }
        s_f[li] = fh;
        const double t = dot2(fx, fy, fx, fy);
        F2 += t;
        M2 = fmax(M2, t);
    }
}

/* Read-only load: through the read-only cache from global memory, or a
 * plain load of a shared-memory copy. */
template <bool RES, class T>
__device__ __forceinline__ T ldro(const T *p) {
    if constexpr (RES) return *p;
    else return __ldg(p);
}

template <int NT, bool RES>
__global__ void __launch_bounds__(NT, 1)
    k_fire_dsm_mixed(const NetDev *nets, const NetDsm *dsms, int n_nets, const int *n_dev, FireParamsDev p,
                     int *queue, const int *order, DsmSizes z, int yield_at, int yield_pm) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ float4 s_dyn[];
    unsigned char *dyn = reinterpret_cast<unsigned char *>(s_dyn);
    const DsmLayout L = dsm_layout(z);
    constexpr bool R = RES;
    float4 *s_u = reinterpret_cast<float4 *>(dyn + L.u); /* {hi.x, hi.y, lo.x, lo.y} */
    float4 *s_tdf = reinterpret_cast<float4 *>(dyn + L.tdf);
    float2 *s_v = reinterpret_cast<float2 *>(dyn + L.v);
    float2 *s_f = reinterpret_cast<float2 *>(dyn + L.f);
    float2 *s_bdf = reinterpret_cast<float2 *>(dyn + L.bdf);
    DsmRes res{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (R)
        res = DsmRes{reinterpret_cast<float4 *>(dyn + L.mb), reinterpret_cast<float4 *>(dyn + L.arms),
                     reinterpret_cast<float2 *>(dyn + L.sk), reinterpret_cast<float2 *>(dyn + L.pk),
                     reinterpret_cast<float2 *>(dyn + L.fahi), reinterpret_cast<float2 *>(dyn + L.falo)};
    int4 *s_tref = reinterpret_cast<int4 *>(dyn + L.tref);
    int2 *s_bref = reinterpret_cast<int2 *>(dyn + L.bref);
    int4 *s_grec = reinterpret_cast<int4 *>(dyn + L.grec);
    int *s_bent = reinterpret_cast<int *>(dyn + L.bent);
    int *s_tent = reinterpret_cast<int *>(dyn + L.tent);
    __shared__ MixShared sh;
    __shared__ NetDev s_d;
    __shared__ NetDsm s_m;
    __shared__ int s_slot;
    /* every CTA's step totals and rank 0's escalation flag, pushed into
     * every CTA of the cluster before the barrier that ends the step: each
     * CTA then reads them from its own shared memory */
    __shared__ float s_parts[kDsmParts][5];
    __shared__ int s_yield_all;
    __shared__ double s_ancs[kDsmParts][2]; /* every CTA's FP64 anchor totals (pushed) */
    __shared__ int s_flag;  /* network start: resume a yielded network; in the loop: leave after this anchor */
    __shared__ unsigned s_au[kDsmParts], s_ab[kDsmParts], s_at[kDsmParts];
    const int rank = (int)cl.block_rank(), C = (int)cl.num_blocks();
    const int spr = kDsmParts / C, lg = __ffs(spr) - 1; /* sub-blocks per CTA, log2 */
    if ((int)threadIdx.x < C) {
        s_au[threadIdx.x] = dsm_addr(s_u, threadIdx.x);
        s_ab[threadIdx.x] = dsm_addr(s_bdf, threadIdx.x);
        s_at[threadIdx.x] = dsm_addr(s_tdf, threadIdx.x);
    }
    /* n_dev: the count of this launch's networks, written on the device by
     * an earlier kernel (device-side escalation); the escalation threshold
     * is then yield_pm / 1000 of the clusters that get a network */
    if (n_dev && yield_pm > 0) {
        const int n_eff = *(volatile const int *)n_dev, clusters = (int)(gridDim.x / C);
        yield_at = max(1, yield_pm * min(clusters, n_eff) / 1000);
    }
    bool ran = false; /* this cluster relaxed a network in this launch */
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) {
            const int sl = atomicAdd(queue, 1);
            s_slot = n_dev && sl >= *(volatile const int *)n_dev ? n_nets : sl;
        }
        cl.sync();
        const int slot = *cl.map_shared_rank(&s_slot, 0);
        /* every CTA has read rank 0's slot before any CTA may exit (a CTA's
         * shared memory must not be read remotely after it exits) or rank 0
         * overwrites it for the next network */
        cl.sync();
        if (slot >= n_nets) {
            /* one more idle cluster (one that never got a network does not
             * count: it was never busy) */
            if (rank == 0 && threadIdx.x == 0 && (ran || !n_dev)) atomicAdd(queue + 1, 1);
            return;
        }
        ran = true;
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
        const int eb0 = m.be[rank * spr], eb1 = m.be[(rank + 1) * spr];
        const int et0 = m.te[rank * spr], et1 = m.te[(rank + 1) * spr];
        if (R) { /* the CTA's read-only slices into shared memory */
            for (int k = threadIdx.x; k < nloc; k += NT) s_grec[k] = m.grec[n0 + k];
            for (int k = threadIdx.x; k < eb1 - eb0; k += NT) s_bent[k] = m.bent[eb0 + k];
            for (int k = threadIdx.x; k < et1 - et0; k += NT) s_tent[k] = m.tent[et0 + k];
            if (d.use_bonds)
                for (int k = threadIdx.x; k < b1 - b0; k += NT) s_bref[k] = m.bref[b0 + k];
            if (d.use_triples)
                for (int k = threadIdx.x; k < t1 - t0; k += NT) s_tref[k] = m.tref[t0 + k];
        }
        /* item and node data for the step loops: shared copies or global */
        const int2 *Bref = R ? s_bref : m.bref + b0;
        const float4 *Mb = R ? res.mb : d.mb_data + b0;
        const float2 *Sk = R ? res.sk : d.mb_sk + b0;
        const int4 *Tref = R ? s_tref : m.tref + t0;
        const float4 *Arms = R ? res.arms : d.mt_arms + t0;
        const float2 *Pk = R ? res.pk : d.mt_pk + t0;
        const int4 *Gr = R ? s_grec : m.grec + n0;
        const int *Be = R ? s_bent : m.bent + eb0;
        const int *Te = R ? s_tent : m.tent + et0;
        const float2 *FaH = R ? res.fahi : d.fa_hi + n0;
        const float2 *FaL = R ? res.falo : d.fa_lo + n0;
        if (threadIdx.x == 0) s_flag = ((volatile FireState *)d.st)->yielded;
        __syncthreads();
        /* the FIRE scalars, advanced by thread 0 of every CTA (identical
         * copies), in shared memory: registers stay free for the passes */
        __shared__ MixScal s_mix;
        __shared__ MixParams s_mq;
        MixScal &s = s_mix;
        MixParams &q = s_mq;
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
            if (R) {
                if (d.use_bonds)
                    for (int k = threadIdx.x; k < b1 - b0; k += NT) {
                        res.mb[k] = d.mb_data[b0 + k];
                        res.sk[k] = d.mb_sk[b0 + k];
                    }
                if (d.use_triples)
                    for (int k = threadIdx.x; k < t1 - t0; k += NT) {
                        res.arms[k] = d.mt_arms[t0 + k];
                        res.pk[k] = d.mt_pk[t0 + k];
                    }
                for (int li = threadIdx.x; li < nloc; li += NT) {
                    res.fahi[li] = d.fa_hi[n0 + li];
                    res.falo[li] = d.fa_lo[n0 + li];
                }
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
            anchor_eval_dsm(d, m, n0, nloc, b0, b1, t0, t1, s_f, res, F2, M2);
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
                const int nb = b1 - b0;
                int sl = threadIdx.x;
                if (sl < nb) {
                    int2 r = ldro<RES>(Bref + sl);
                    float4 ra = Mb[sl];
                    float2 sk = Sk[sl];
                    for (;;) {
                        const float4 ui = dsm_ld4(u_addr(s_au, r.x, lg, bsub));
                        const float4 uj = dsm_ld4(u_addr(s_au, r.y, lg, bsub));
                        const int nx = sl + NT;
                        int2 rn = r;
                        float4 ran = ra;
                        float2 skn = sk;
                        if (nx < nb) {
                            rn = ldro<RES>(Bref + nx);
                            ran = Mb[nx];
                            skn = Sk[nx];
                        }
                        float2 dh, dlo;
                        u_diff2(make_float2(uj.x, uj.y), make_float2(uj.z, uj.w), make_float2(ui.x, ui.y),
                                make_float2(ui.z, ui.w), dh, dlo);
                        s_bdf[sl] = bond_dforce(ra, sk, dh, dlo);
                        if (nx >= nb) break;
                        sl = nx;
                        r = rn;
                        ra = ran;
                        sk = skn;
                    }
                }
            }
            if (d.use_triples) {
                const int nt = t1 - t0;
                int sl = threadIdx.x;
                if (sl < nt) {
                    int4 r = ldro<RES>(Tref + sl);
                    float4 arms = Arms[sl];
                    float2 pk = Pk[sl];
                    for (;;) {
                        const float4 uh = dsm_ld4(u_addr(s_au, r.x, lg, bsub));
                        const float4 uj = dsm_ld4(u_addr(s_au, r.y, lg, bsub));
                        const float4 uk = dsm_ld4(u_addr(s_au, r.z, lg, bsub));
                        const int nx = sl + NT;
                        int4 rn = r;
                        float4 armsn = arms;
                        float2 pkn = pk;
                        if (nx < nt) {
                            rn = ldro<RES>(Tref + nx);
                            armsn = Arms[nx];
                            pkn = Pk[nx];
                        }
                        const float2 hh = make_float2(uh.x, uh.y), hl = make_float2(uh.z, uh.w);
                        float2 dFj, dFk;
                        tri_dforce(arms, pk, u_diff(make_float2(uj.x, uj.y), make_float2(uj.z, uj.w), hh, hl),
                                   u_diff(make_float2(uk.x, uk.y), make_float2(uk.z, uk.w), hh, hl), dFj, dFk);
                        s_tdf[sl] = make_float4(dFj.x, dFj.y, dFk.x, dFk.y);
                        if (nx >= nt) break;
                        sl = nx;
                        r = rn;
                        arms = armsn;
                        pk = pkn;
                    }
                }
            }
            cl.sync();
            /* gather: F = F(X) + the node's entries in incidence order, half
             * kick; the nodes in gather-record order (lanes of a warp take
             * nodes with equally long entry lists) */
            float P = 0.f, V2 = 0.f, Fs = 0.f, M2f = 0.f, A = 0.f;
            /* rank 0 reads the idle-cluster count now; its global-memory
             * latency passes during the gather instead of before the
             * cluster barrier */
            int idle = 0;
            if (rank == 0 && threadIdx.x == 0 && yield_at > 0) idle = *(volatile int *)(queue + 1);
            for (int k = threadIdx.x; k < nloc; k += NT) {
                /* one record load gives the node, its fcode and both entry
                 * ranges */
                const int4 g = ldro<RES>(Gr + k);
                const int li = (g.x & 0x0fffffff) - n0;
                const unsigned fc = (unsigned)g.x >> 28;
                const int bq0 = g.y - eb0, bq1 = bq0 + (g.z & 0xffff);
                const int tq0 = g.w - et0, tq1 = tq0 + ((unsigned)g.z >> 16);
                const float2 ah = FaH[li], al = FaL[li];
                float2 F = make_float2(0.f, 0.f);
                if (fc != 0) {
                    float2 dF = make_float2(0.f, 0.f);
                    float mag = 0.f;
                    if (d.use_bonds) {
#pragma unroll 4
                        for (int e = bq0; e < bq1; ++e) {
                            const unsigned code = (unsigned)ldro<RES>(Be + e);
                            const int r = (int)(code >> 28) >> lg;
                            const int ls = (int)((code >> 1) & 0x7ffffffu) - s_m.bo[r * spr];
                            float2 df = dsm_ld2(s_ab[r] + 8u * (unsigned)ls);
                            df = neg_if(df, code);
                            dF.x += df.x;
                            dF.y += df.y;
                            mag += fabsf(df.x) + fabsf(df.y);
                        }
                    }
                    if (d.use_triples) {
#pragma unroll 4
                        for (int e = tq0; e < tq1; ++e) {
                            const unsigned code = (unsigned)ldro<RES>(Te + e);
                            const int r = (int)(code >> 28) >> lg;
                            const int role = code & 3;
                            const int ls = (int)((code >> 2) & 0x3ffffffu) - s_m.to[r * spr];
                            const float4 qv = dsm_ld4(s_at[r] + 16u * (unsigned)ls);
                            float gx, gy, mg;
                            tri_entry(qv, role, gx, gy, mg);
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
                /* rank 0's escalation flag: thread 0 read the idle count, so
                 * lane 0's decision goes to every lane before any is pushed
                 * (every CTA must take the same branch) */
                const int yv = __shfl_sync(kFull, (int)(yield_at > 0 && idle >= yield_at), 0);
                /* lane r pushes this CTA's totals into CTA r (remote stores
                 * complete before the cluster barrier releases) */
                if ((int)threadIdx.x < C) {
                    const unsigned a = dsm_addr(&s_parts[rank][0], threadIdx.x);
                    dsm_st1(a, t.P);
                    dsm_st1(a + 4u, t.V2);
                    dsm_st1(a + 8u, t.F2);
                    dsm_st1(a + 12u, t.M2);
                    dsm_st1(a + 16u, t.A);
                    if (rank == 0) dsm_st1i(dsm_addr(&s_yield_all, threadIdx.x), yv);
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
                    /* rank 0's escalation flag, the same in every CTA */
                    const int y = s_yield_all;
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
                anchor_eval_dsm(d, m, n0, nloc, b0, b1, t0, t1, s_f, res, F2, M2);
                anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
                if (threadIdx.x == 0) anchor_push(s_ancs, rank, C, tF2, tM2);
                cl.sync();
                if (threadIdx.x == 0) {
                    double t[2];
                    anchor_totals(s_ancs, C, t);
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
size_t dsm_smem_bytes(int bmax, int emax, int tmax, int ebmax, int etmax, int resident) {
    return dsm_layout(DsmSizes{bmax, emax, tmax, ebmax, etmax, resident}).total;
}

/* Largest dynamic shared memory the kernel may use on this device. */
size_t dsm_smem_limit() {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, (const void *)k_fire_dsm_mixed<512, true>) != cudaSuccess) return 0;
    return optin > (int)fa.sharedSizeBytes ? (size_t)(optin - (int)fa.sharedSizeBytes) : 0;
}

template <int NT, bool RES>
static cudaError_t dsm_config(int cluster, const DsmSizes &z, cudaLaunchConfig_t &cfg, cudaLaunchAttribute *attr,
                              int *max_clusters) {
    cudaError_t e;
    int dev, sms;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const size_t smem = dsm_layout(z).total;
    if ((e = cudaFuncSetAttribute(k_fire_dsm_mixed<NT, RES>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return e;
    if (cluster > 8 &&
        (e = cudaFuncSetAttribute(k_fire_dsm_mixed<NT, RES>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) !=
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
    return cudaOccupancyMaxActiveClusters(max_clusters, (void *)k_fire_dsm_mixed<NT, RES>, &cfg);
}

template <int NT, bool RES>
static cudaError_t launch_dsm_nt(const NetDev *nets_dev, const NetDsm *dsm_dev, int n_nets, const int *n_dev,
                                 int cluster, const DsmSizes &z, double escalate, int cap, const FireParamsDev &p,
                                 int *queue_dev, const int *order_dev, cudaStream_t stream) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    int max_clusters = 0;
    cudaError_t e = dsm_config<NT, RES>(cluster, z, cfg, attr, &max_clusters);
    if (e != cudaSuccess) return e;
    if (max_clusters < 1) return cudaErrorLaunchOutOfResources;
    int clusters = std::max(1, std::min(n_nets, max_clusters));
    if (cap > 0) clusters = std::min(clusters, cap);
    cfg.gridDim = dim3(clusters * cluster);
    cfg.stream = stream;
    const int yield_at = escalate > 0 ? std::max(1, (int)(escalate * clusters)) : 0;
    const int yield_pm = escalate > 0 ? std::max(1, (int)(1000.0 * escalate)) : 0;
    if ((e = cudaMemsetAsync(queue_dev, 0, 2 * sizeof(int), stream)) != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, k_fire_dsm_mixed<NT, RES>, nets_dev, dsm_dev, n_nets, n_dev, p, queue_dev,
                              order_dev, z, yield_at, n_dev ? yield_pm : 0);
}

/* Threads per CTA: NR_MIX_THREADS (512 or 1024), else 1024 when the state
 * fills shared memory (many items per thread: more warps hide more
 * latency) and 512 when the CTA is resident (few items per thread: the
 * 128-register budget keeps the step free of spills). */
static int dsm_threads(bool resident) {
    const char *env = knob("NR_MIX_THREADS");
    if (env && (atoi(env) == 512 || atoi(env) == 1024)) return atoi(env);
    return resident ? 512 : 1024;
}

cudaError_t launch_mixed_dsm(const NetDev *nets_dev, const NetDsm *dsm_dev, int n_nets, int cluster, int bmax,
                             int emax, int tmax, int ebmax, int etmax, int resident, double escalate, int cap,
                             const FireParamsDev &p, int *queue_dev, const int *order_dev, cudaStream_t stream,
                             const int *n_dev) {
    if (cluster < 1 || cluster > kDsmParts || (kDsmParts % cluster) != 0) return cudaErrorInvalidValue;
    const DsmSizes z{bmax, emax, tmax, ebmax, etmax, resident};
    const bool wide = dsm_threads(resident != 0) == 1024;
    if (resident)
        return wide ? launch_dsm_nt<1024, true>(nets_dev, dsm_dev, n_nets, n_dev, cluster, z, escalate, cap, p,
                                                queue_dev, order_dev, stream)
                    : launch_dsm_nt<512, true>(nets_dev, dsm_dev, n_nets, n_dev, cluster, z, escalate, cap, p,
                                               queue_dev, order_dev, stream);
    return wide ? launch_dsm_nt<1024, false>(nets_dev, dsm_dev, n_nets, n_dev, cluster, z, escalate, cap, p, queue_dev,
                                             order_dev, stream)
                : launch_dsm_nt<512, false>(nets_dev, dsm_dev, n_nets, n_dev, cluster, z, escalate, cap, p, queue_dev,
                                            order_dev, stream);
}

/* Device-side escalation: the networks of a batch that left their last
 * launch at an anchor (FireState.yielded), in index order, into order_out,
 * and their count into *count_out.  One CTA; a block-wide scan per chunk of
 * blockDim networks. */
__global__ void k_compact_yielded(const FireState *st, int n, int *order_out, int *count_out) {
    __shared__ int s_warp[32];
    __shared__ int s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    for (int c0 = 0; c0 < n; c0 += blockDim.x) {
        const int i = c0 + threadIdx.x;
        const int flag = i < n && ((volatile const FireState *)st)[i].yielded ? 1 : 0;
        const unsigned bal = __ballot_sync(kFull, flag);
        const int in_warp = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        int before = s_base;
        for (int w = 0; w < warp; ++w) before += s_warp[w];
        if (flag) order_out[before + in_warp] = i;
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 0; w < nw; ++w) s_base += s_warp[w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *count_out = s_base;
}

cudaError_t launch_compact_yielded(const FireState *st, int n, int *order_out, int *count_out, cudaStream_t stream) {
    k_compact_yielded<<<1, 256, 0, stream>>>(st, n, order_out, count_out);
    return cudaGetLastError();
}

cudaError_t dsm_max_active(int cluster, int bmax, int emax, int tmax, int ebmax, int etmax, int resident, int *out) {
    const DsmSizes z{bmax, emax, tmax, ebmax, etmax, resident};
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    const bool wide = dsm_threads(resident != 0) == 1024;
    if (resident)
        return wide ? dsm_config<1024, true>(cluster, z, cfg, attr, out) : dsm_config<512, true>(cluster, z, cfg, attr, out);
    return wide ? dsm_config<1024, false>(cluster, z, cfg, attr, out) : dsm_config<512, false>(cluster, z, cfg, attr, out);
}

}  // namespace nr
