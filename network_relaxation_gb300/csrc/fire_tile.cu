/*
 * Mixed-precision FIRE for one large network over the whole GPU, in spatial
 * tiles, with ONE grid barrier per FIRE step and every tile's read-only data
 * streamed into shared memory by TMA bulk copies.
 *
 * The cooperative grid kernel of fire_mixed.cu runs a step as four passes
 * separated by grid barriers (drift, item pass writing every bond's and
 * triple's FP32 force change to global memory, gather reading them back,
 * reduction by the last CTA); it is bound by the latency of those passes and
 * barriers.  Here one CTA per SM takes whole tiles (NetTile, nr_device.cuh)
 * and does a tile's whole step on chip:
 *   0. the tile's record (item references, anchor records, incidence,
 *      fcodes, halo list: one contiguous block) arrives in shared memory by
 *      one cp.async.bulk, issued while the previous tile computes (two
 *      stage buffers, an mbarrier each);
 *   1. u, v, F of the own nodes (contiguous in tile order) and of the halo;
 *   2. pass A (mixing, drift, half kick) for own AND halo nodes: the halo's
 *      drift is recomputed from the same inputs with the same operations as
 *      its owner's, so it has the same bits and needs no barrier;
 *   3. the item pass: every bond's and triple's FP32 force change into
 *      shared memory (boundary items are evaluated by each tile they touch);
 *   4. the gather of the own nodes in the canonical incidence order, half
 *      kick, the next step's u, v, F written, the step's partial sums.
 * Then one grid barrier; every CTA combines the CTAs' partials in CTA order
 * itself and advances an identical copy of the FIRE scalars.  The
 * arithmetic (double-float u, bond_dforce, tri_dforce, FP32 FIRE step, FP64
 * anchors and certification) is mixed_common.cuh's; per node the force is
 * the same sum in the same order as in the other mixed kernels.  Anchors
 * (rare) take two more barriers: X += u, then the FP64 force and the tile
 * records' anchor data.
 *
 * Every wait is bounded: the grid barrier by a %globaltimer budget, the
 * mbarrier waits by the same budget; a wait that runs out sets the
 * network's abort flag (NR_ERR_TIMEOUT on the host), waits (bounded) for the
 * CTA's copy in flight, and returns.
 *
 * Compiled with --fmad=false; FP32 expressions use explicit fmaf().
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fire_launch.h"
#include "mixed_common.cuh"
#include "nr_internal.h"

namespace nr {

/* ----- grid barrier: a monotonic counter, every CTA waits for all ----- */

/* Arrives at barrier number `epoch` (1, 2, ...) of the launch and waits
 * until all G CTAs have; false when the wait exceeded budget_ns or another
 * CTA gave up (st->abort_flag); every thread of the CTA sees the same
 * result. */
__device__ inline bool tile_barrier(const NetTile &tl, FireState *st, unsigned G, unsigned long long epoch,
                                    unsigned long long budget_ns, unsigned site) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        atomicAdd(tl.bar, 1ULL);
        const unsigned long long target = epoch * (unsigned long long)G;
        volatile unsigned long long *bar = tl.bar;
        volatile unsigned *abort_flag = &st->abort_flag;
        const unsigned long long t0 = global_ns();
        unsigned spins = 0;
        while (*bar < target) {
            if (*abort_flag) {
                ok = 0;
                break;
            }
            if ((++spins & 63u) == 0 && global_ns() - t0 > budget_ns) {
                atomicExch(&st->abort_flag, 1u);
                atomicExch(&st->timeout_site, site);
                ok = 0;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    const int ok = s_ok;
    __syncthreads();
    return ok != 0;
}

/* ----- TMA bulk copy into shared memory, completion on an mbarrier ----- */

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(mbar)));
}

/* One thread: expect `bytes` and copy them from global src to shared dst
 * (both 16-byte aligned, bytes a multiple of 16: the host checks the
 * layout). */
__device__ __forceinline__ void tma_load(void *dst, const void *src, unsigned bytes, unsigned long long *mbar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(mbar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long *mbar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(mbar)), "r"(parity)
        : "memory");
    return ok != 0;
}

/* Waits (every thread) until the mbarrier's phase `parity` completed, at
 * most budget_ns; false when it ran out. */
__device__ inline bool mbar_wait(unsigned long long *mbar, unsigned parity, unsigned long long budget_ns) {
    if (mbar_try_wait(mbar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned spins = 0;; ++spins) {
        if (mbar_try_wait(mbar, parity)) return true;
        if ((spins & 15u) == 15u && global_ns() - t0 > budget_ns) return false;
    }
}

/* ----- per-thread asynchronous copies into shared memory (cp.async) ----- */

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

/* ----- per-tile pieces ----- */

/* A tile's node state in shared memory: u, v, F of its own nodes (local 0
 * .. no - 1) and halo nodes (no .. no + nh - 1), the own nodes' anchor
 * force.  Two of them: the next tile's state is copied in while the current
 * tile computes. */
struct TileState {
    float4 *u;  /* double-float u {hi.x, hi.y, lo.x, lo.y} */
    float4 *vf; /* {v.x, v.y, F.x, F.y} */
    float4 *fa; /* own nodes: double-float anchor force {hi.x, hi.y, lo.x, lo.y} */
};
__host__ __device__ inline size_t tile_state_bytes(int max_nodes, int max_own) {
    return 32 * (size_t)max_nodes + 16 * (size_t)max_own;
}
__device__ inline TileState tile_state_at(unsigned char *base, int max_nodes, int max_own) {
    TileState t;
    t.u = reinterpret_cast<float4 *>(base);
    t.vf = t.u + max_nodes;
    t.fa = t.vf + max_nodes;
    return t;
}

/* Starts the copies of tile td's own state (state copy `cur`). */
__device__ __forceinline__ void issue_own(const NetTile &tl, const TileDesc &td, int cur, const TileState &ts) {
    for (int k = threadIdx.x; k < td.no; k += blockDim.x) {
        const int p = td.own_pos + k;
        cp_async16(ts.u + k, tl.u[cur] + p);
        cp_async16(ts.vf + k, tl.vf[cur] + p);
        cp_async16(ts.fa + k, tl.fa + p);
    }
}
/* Starts the copies of tile td's halo state (its record already in shared
 * memory). */
__device__ __forceinline__ void issue_halo(const NetTile &tl, const TileDesc &td, const unsigned char *rec, int cur,
                                           const TileState &ts) {
    const TileSegs g = tile_segs(td.nb, td.nt, td.no, td.ni, td.nh);
    const int *halo = reinterpret_cast<const int *>(rec + g.halo);
    for (int h = threadIdx.x; h < td.nh; h += blockDim.x) {
        const int pp = halo[h];
        cp_async16(ts.u + td.no + h, tl.u[cur] + pp);
        cp_async16(ts.vf + td.no + h, tl.vf[cur] + pp);
    }
}

/* Pass A of one node (mixed_pass_a's operations). */
__device__ __forceinline__ void tile_pass_a(const Coef &c, float4 &w, float2 &v, const float2 F) {
    if (c.mix_pending) {
        v.x = fmaf(c.na, v.x, v.x);
        v.y = fmaf(c.na, v.y, v.y);
        v.x = fmaf(c.a, F.x, v.x);
        v.y = fmaf(c.a, F.y, v.y);
        if (c.zero_v) v = make_float2(0.f, 0.f);
    }
    if (!c.done) {
        df_add(w.x, w.z, fmaf(c.dt, v.x, c.dtsq * F.x));
        df_add(w.y, w.w, fmaf(c.dt, v.y, c.dtsq * F.y));
        v.x = fmaf(c.dtm, F.x, v.x);
        v.y = fmaf(c.dtm, F.y, v.y);
    }
}

/* FP64 anchor evaluation: X += u was done; every node's canonical FP64
 * force (d.f), its double-float copy fa and F = fa_hi in the current state
 * copy (tile order); the anchor data of the CTA's tiles' records.  Returns
 * the CTA partials of |F|^2 (sum) and max |F|^2 in thread 0. */
static __device__ __noinline__ void tile_anchor_eval(const NetDev &d, const NetTile &tl, int cur, double *dslots,
                                                     double &tF2, double &tM2) {
    const double W = d.width;
    double F2 = 0.0, M2 = 0.0;
    const int G = gridDim.x;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < tl.n_pos; p += G * blockDim.x) {
        const int i = tl.node_of_pos[p];
        if (i < 0) continue;
        double fx, fy;
        node_force_fp64_own<false>(d, i, fx, fy);
        d.f[i] = make_double2(fx, fy);
        const float hx = (float)fx, hy = (float)fy;
        tl.fa[p] = make_float4(hx, hy, (float)(fx - (double)hx), (float)(fy - (double)hy));
        float4 q = tl.vf[cur][p]; /* v stays, F = the anchor force */
        q.z = hx;
        q.w = hy;
        tl.vf[cur][p] = q;
        const double t = dot2(fx, fy, fx, fy);
        F2 += t;
        M2 = fmax(M2, t);
    }
    for (int t = blockIdx.x; t < tl.n_tiles; t += G) {
        const TileDesc td = tl.desc[t];
        const TileSegs g = tile_segs(td.nb, td.nt, td.no, td.ni, td.nh);
        unsigned char *rec = tl.ro + td.ro_off;
        float4 *mb = reinterpret_cast<float4 *>(rec + g.mb);
        float2 *sk = reinterpret_cast<float2 *>(rec + g.sk);
        float4 *arms = reinterpret_cast<float4 *>(rec + g.arms);
        float2 *pk = reinterpret_cast<float2 *>(rec + g.pk);
        if (d.use_bonds)
            for (int k = threadIdx.x; k < td.nb; k += blockDim.x) {
                const int b = tl.bid[td.bond_off + k];
                const int4 r = d.bond[b];
                const double2 p1 = d.x[r.x], p2 = d.x[r.y];
                const double rx = (p2.x + wrap_shift(r.z, W)) - p1.x, ry = p2.y - p1.y;
                const double kk = d.bond_k ? d.bond_k[b] : d.ks;
                const float hx = (float)rx, hy = (float)ry;
                mb[k] = make_float4(hx, hy, (float)(rx - (double)hx), (float)(ry - (double)hy));
                sk[k] = make_float2((float)(sqrt(fma(rx, rx, ry * ry)) - d.bond_l0[b]), (float)kk);
            }
        if (d.use_triples)
            for (int k = threadIdx.x; k < td.nt; k += blockDim.x) {
                const int tt = tl.tid[td.tri_off + k];
                const int4 r = d.tri[tt];
                const double2 ph = d.x[r.x], pj = d.x[r.y], pkk = d.x[r.z];
                const int wj = (signed char)(r.w & 0xff), wk = (signed char)((r.w >> 8) & 0xff);
                const double ax = (pj.x + wrap_shift(wj, W)) - ph.x, ay = pj.y - ph.y;
                const double bx = (pkk.x + wrap_shift(wk, W)) - ph.x, by = pkk.y - ph.y;
                const double kb = d.tri_kb ? d.tri_kb[tt] : d.kb;
                const double phi0 = d.tri_phi0 ? d.tri_phi0[tt] : 0.0;
                arms[k] = make_float4((float)ax, (float)ay, (float)bx, (float)by);
                pk[k] = make_float2((float)bend_dtheta(ax, ay, bx, by, phi0), (float)kb);
            }
    }
    /* the records are read later by bulk copies (the async proxy) */
    asm volatile("fence.proxy.async.global;" ::: "memory");
    anchor_reduce(F2, M2, dslots, tF2, tM2);
}

/* Totals of the CTAs' FP64 anchor partials, in CTA order (thread 0). */
static __device__ __noinline__ void tile_anchor_totals(const NetTile &tl, int G, double &F2, double &M2) {
    double s = 0.0, m = 0.0;
    for (int c = 0; c < G; ++c) {
        s = s + __ldcg(tl.dpart + 2 * c);
        m = fmax(m, __ldcg(tl.dpart + 2 * c + 1));
    }
    F2 = s;
    M2 = m;
}

/* Instantiated for 512 or 768 threads per CTA with one CTA per SM (768: more
 * warps to hide latency, fewer registers per thread), and for 256 threads
 * with two CTAs per SM (smaller tiles; one CTA's barriers overlap the
 * other's work). */

/* Dynamic shared memory of a CTA: two record buffers of max_ro bytes, two
 * node-state buffers, the item results of one tile. */
__host__ __device__ inline size_t tile_smem_bytes(unsigned max_ro, int max_nodes, int max_own, int max_bonds,
                                                  int max_tris) {
    return 2 * (size_t)max_ro + 2 * tile_state_bytes(max_nodes, max_own) + 16 * (size_t)max_tris +
           8 * (size_t)max_bonds;
}

constexpr int kDescCache = 32;

template <int NT, int MINB>
__global__ void __launch_bounds__(NT, MINB)
    k_fire_tile_mixed(NetDev d, NetTile tl, FireParamsDev p, unsigned long long budget_ns) {
    extern __shared__ float4 s_dyn[];
    __shared__ MixShared sh;
    __shared__ __align__(8) unsigned long long s_mbar[2];
    __shared__ int s_fail;
    /* FIRE scalars, advanced by thread 0 of every CTA (identical copies) */
    __shared__ MixScal s;
    __shared__ MixParams q;
    /* the descriptors of the CTA's first kDescCache tiles, loaded once: a
     * tile's first instructions then wait on shared memory, not on L2 */
    __shared__ TileDesc s_desc[kDescCache];
    unsigned char *dyn = reinterpret_cast<unsigned char *>(s_dyn);
    unsigned char *const stage0 = dyn, *const stage1 = dyn + tl.max_ro;
    const size_t sbytes = tile_state_bytes(tl.max_nodes, tl.max_own);
    const TileState ts0 = tile_state_at(dyn + 2 * (size_t)tl.max_ro, tl.max_nodes, tl.max_own);
    const TileState ts1 = tile_state_at(dyn + 2 * (size_t)tl.max_ro + sbytes, tl.max_nodes, tl.max_own);
    float4 *s_tdf = reinterpret_cast<float4 *>(dyn + 2 * (size_t)tl.max_ro + 2 * sbytes);
    float2 *s_bdf = reinterpret_cast<float2 *>(s_tdf + tl.max_tris);
    const unsigned G = gridDim.x;
    FireState *st = d.st;
    unsigned long long epoch = 0;
    unsigned uses0 = 0u, uses1 = 0u; /* completed phases of each stage buffer's mbarrier */
    unsigned iss0 = 0u, iss1 = 0u;   /* record copies issued into each stage buffer */
    if (threadIdx.x == 0) {
        q = mix_params(p, d.sqrt_dof);
        mbar_init(&s_mbar[0]);
        mbar_init(&s_mbar[1]);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_fail = 0;
    }
    __syncthreads();
    int cur = 0;
    for (int i = blockIdx.x * NT + threadIdx.x; i < tl.n_pos; i += G * NT) {
        tl.u[0][i] = make_float4(0.f, 0.f, 0.f, 0.f);
        tl.vf[0][i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    double tF2, tM2;
    tile_anchor_eval(d, tl, cur, sh.dslots, tF2, tM2);
    if (threadIdx.x == 0) {
        tl.dpart[2 * blockIdx.x] = tF2;
        tl.dpart[2 * blockIdx.x + 1] = tM2;
    }
    if (!tile_barrier(tl, st, G, ++epoch, budget_ns, 21)) return;
    if (threadIdx.x == 0) {
        double F2, M2;
        tile_anchor_totals(tl, G, F2, M2);
        mix_init(s, q);
        mix_certify(s, p, d.sqrt_dof, F2, M2);
        sh.coef = coef_of(s, 0);
    }
    __syncthreads();
    const int n_mine = (int)blockIdx.x < tl.n_tiles ? (tl.n_tiles - 1 - (int)blockIdx.x) / (int)G + 1 : 0;
    for (int k = threadIdx.x; k < min(n_mine, kDescCache); k += NT) s_desc[k] = tl.desc[blockIdx.x + k * G];
    __syncthreads();
    auto desc = [&](int k) -> TileDesc { return k < kDescCache ? s_desc[k] : tl.desc[blockIdx.x + k * G]; };
    for (;;) {
        const Coef &c = sh.coef;
        if (c.done) {
            /* the last pass A: mixing of v only (u is 0 after the certifying
             * anchor); the FP64 velocities out */
            for (int pp = blockIdx.x * NT + threadIdx.x; pp < tl.n_pos; pp += G * NT) {
                const int i = tl.node_of_pos[pp];
                if (i < 0) continue;
                float4 w = tl.u[cur][pp];
                const float4 q = tl.vf[cur][pp];
                float2 v = make_float2(q.x, q.y);
                tile_pass_a(c, w, v, make_float2(q.z, q.w));
                d.v[i] = make_double2((double)v.x, (double)v.y);
            }
            break;
        }
        const int nxt = cur ^ 1;
        float P = 0.f, V2 = 0.f, Fs = 0.f, M2f = 0.f, A = 0.f;
        /* the pipeline: the record (TMA) and the node state (cp.async) of
         * tile k + 1 are in flight while tile k computes */
        if (n_mine > 0) {
            const TileDesc td0 = desc(0);
            if (threadIdx.x == 0)
                tma_load(stage0, tl.ro + td0.ro_off, tile_segs(td0.nb, td0.nt, td0.no, td0.ni, td0.nh).total,
                         &s_mbar[0]);
            ++iss0;
            issue_own(tl, td0, cur, ts0);
            cp_async_commit();
            if (mbar_wait(&s_mbar[0], uses0 & 1u, budget_ns)) {
                ++uses0;
                issue_halo(tl, td0, stage0, cur, ts0); /* only from a record that arrived */
            } else {
                s_fail = 1;
            }
            cp_async_commit();
        }
        /* a wait that ran out: record the timeout, let every copy in flight
         * land (record copies: bounded waits), leave */
        auto abort_tiles = [&]() {
            if (threadIdx.x == 0) {
                atomicExch(&st->abort_flag, 1u);
                atomicExch(&st->timeout_site, 25u);
            }
            cp_async_wait_all();
            if (iss0 > uses0) mbar_wait(&s_mbar[0], uses0 & 1u, budget_ns);
            if (iss1 > uses1) mbar_wait(&s_mbar[1], uses1 & 1u, budget_ns);
        };
        for (int k = 0; k < n_mine; ++k) {
            const int b = k & 1;
            const TileDesc td = desc(k);
            const bool more = k + 1 < n_mine;
            const TileDesc tn = more ? desc(k + 1) : td;
            const TileState &sc = b ? ts1 : ts0, &sn = b ? ts0 : ts1;
            unsigned char *const rec_n = b ? stage0 : stage1;
            __syncthreads();
            if (s_fail) {
                abort_tiles();
                return;
            }
            if (more) {
                if (threadIdx.x == 0)
                    tma_load(rec_n, tl.ro + tn.ro_off, tile_segs(tn.nb, tn.nt, tn.no, tn.ni, tn.nh).total,
                             &s_mbar[b ^ 1]);
                if (b) ++iss0;
                else ++iss1;
                issue_own(tl, tn, cur, sn);
            }
            cp_async_commit();
            cp_async_wait1(); /* this tile's own and halo state is in */
            __syncthreads();
            const TileSegs g = tile_segs(td.nb, td.nt, td.no, td.ni, td.nh);
            const int no = td.no, nn = no + td.nh, op = td.own_pos;
            const unsigned char *rec = b ? stage1 : stage0;
            /* pass A of own and halo nodes, in place */
            for (int kk = threadIdx.x; kk < nn; kk += NT) {
                float4 w = sc.u[kk];
                const float4 q = sc.vf[kk];
                float2 v = make_float2(q.x, q.y);
                tile_pass_a(c, w, v, make_float2(q.z, q.w));
                sc.u[kk] = w;
                sc.vf[kk] = make_float4(v.x, v.y, q.z, q.w);
            }
            __syncthreads();
            /* item pass into shared memory */
            if (d.use_bonds) {
                const unsigned *bref = reinterpret_cast<const unsigned *>(rec + g.bref);
                const float4 *mb = reinterpret_cast<const float4 *>(rec + g.mb);
                const float2 *sk = reinterpret_cast<const float2 *>(rec + g.sk);
                for (int kk = threadIdx.x; kk < td.nb; kk += NT) {
                    const unsigned r = bref[kk];
                    const float4 ui = sc.u[r & 0xffffu], uj = sc.u[r >> 16];
                    float2 dh, dlo;
                    u_diff2(make_float2(uj.x, uj.y), make_float2(uj.z, uj.w), make_float2(ui.x, ui.y),
                            make_float2(ui.z, ui.w), dh, dlo);
                    s_bdf[kk] = bond_dforce(mb[kk], sk[kk], dh, dlo);
                }
            }
            if (d.use_triples) {
                const uint2 *tref = reinterpret_cast<const uint2 *>(rec + g.tref);
                const float4 *arms = reinterpret_cast<const float4 *>(rec + g.arms);
                const float2 *pk = reinterpret_cast<const float2 *>(rec + g.pk);
                for (int kk = threadIdx.x; kk < td.nt; kk += NT) {
                    const uint2 r = tref[kk];
                    const float4 uh = sc.u[r.x & 0xffffu], uj = sc.u[r.x >> 16], uk = sc.u[r.y];
                    const float2 hh = make_float2(uh.x, uh.y), hl = make_float2(uh.z, uh.w);
                    float2 dFj, dFk;
                    tri_dforce(arms[kk], pk[kk], u_diff(make_float2(uj.x, uj.y), make_float2(uj.z, uj.w), hh, hl),
                               u_diff(make_float2(uk.x, uk.y), make_float2(uk.z, uk.w), hh, hl), dFj, dFk);
                    s_tdf[kk] = make_float4(dFj.x, dFj.y, dFk.x, dFk.y);
                }
            }
            /* the next tile's record is in by now (bounded wait): start its
             * halo state */
            if (more) {
                if (mbar_wait(&s_mbar[b ^ 1], (b ? uses0 : uses1) & 1u, budget_ns)) {
                    if (b) ++uses0;
                    else ++uses1;
                    issue_halo(tl, tn, rec_n, cur, sn); /* only from a record that arrived */
                } else {
                    s_fail = 1;
                }
            }
            cp_async_commit();
            __syncthreads();
            if (s_fail) {
                abort_tiles();
                return;
            }
            /* gather of the own nodes, half kick, the next step's state */
            const unsigned short *iptr = reinterpret_cast<const unsigned short *>(rec + g.iptr);
            const unsigned short *ibe = reinterpret_cast<const unsigned short *>(rec + g.ibe);
            const unsigned short *inc = reinterpret_cast<const unsigned short *>(rec + g.inc);
            const unsigned char *fcode = rec + g.fcode;
            for (int kk = threadIdx.x; kk < no; kk += NT) {
                const unsigned fc = fcode[kk];
                const int e0 = iptr[kk], eb = ibe[kk], e1 = iptr[kk + 1];
                const float4 fa = sc.fa[kk];
                const float2 ah = make_float2(fa.x, fa.y), al = make_float2(fa.z, fa.w);
                float2 F = make_float2(0.f, 0.f);
                if (fc != 0) {
                    /* the node's bond entries, then its triple entries (the
                     * canonical order), each list without a branch per
                     * entry; own nodes are ordered by list lengths */
                    float2 dF = make_float2(0.f, 0.f);
                    float mag = 0.f;
#pragma unroll 4
                    for (int e = e0; e < eb; ++e) {
                        const unsigned code = inc[e];
                        float2 df = s_bdf[code >> 1];
                        df = neg_if(df, code);
                        dF.x += df.x;
                        dF.y += df.y;
                        mag += fabsf(df.x) + fabsf(df.y);
                    }
#pragma unroll 4
                    for (int e = eb; e < e1; ++e) {
                        const unsigned code = inc[e];
                        const int role = code & 3;
                        const float4 qv = s_tdf[(code & 0x7fffu) >> 2];
                        float gx, gy, mg;
                        tri_entry(qv, role, gx, gy, mg);
                        dF.x += gx;
                        dF.y += gy;
                        mag += mg;
                    }
                    A = fmaxf(A, mag);
                    F.x = ah.x + (al.x + dF.x);
                    F.y = ah.y + (al.y + dF.y);
                    if (!(fc & 1)) F.x = 0.f;
                    if (!(fc & 2)) F.y = 0.f;
                }
                const float4 q = sc.vf[kk];
                float2 v = make_float2(q.x, q.y);
                v.x = fmaf(c.dtm, F.x, v.x);
                v.y = fmaf(c.dtm, F.y, v.y);
                tl.u[nxt][op + kk] = sc.u[kk];
                tl.vf[nxt][op + kk] = make_float4(v.x, v.y, F.x, F.y);
                P += fmaf(v.x, F.x, v.y * F.y);
                V2 += fmaf(v.x, v.x, v.y * v.y);
                const float f2 = fmaf(F.x, F.x, F.y * F.y);
                Fs += f2;
                M2f = fmaxf(M2f, f2);
            }
            /* the next tile's first barrier orders this gather's reads of the
             * stage and state buffers before they are refilled */
        }
        cp_async_wait_all();
        warp_part(Part{P, V2, Fs, M2f, A}, sh.slots);
        __syncthreads();
        if (threadIdx.x < 32) {
            const Part t = block_totals(sh.slots);
            if (threadIdx.x == 0) {
                /* two copies by step parity: a CTA that runs ahead into the
                 * next step writes the other copy while the rest still read
                 * this one */
                float *cp = tl.cpart + 5 * ((size_t)cur * G + blockIdx.x);
                cp[0] = t.P;
                cp[1] = t.V2;
                cp[2] = t.F2;
                cp[3] = t.M2;
                cp[4] = t.A;
            }
        }
        if (!tile_barrier(tl, st, G, ++epoch, budget_ns, 22)) return;
        if (threadIdx.x < 32) {
            /* lane l accumulates CTAs l, l + 32, ... in order, then the
             * butterfly: the same totals in every CTA */
            Part t{0.f, 0.f, 0.f, 0.f, 0.f};
            for (int kk = threadIdx.x; kk < (int)G; kk += 32) {
                const float *cp = tl.cpart + 5 * ((size_t)cur * G + kk);
                t.P += __ldcg(cp);
                t.V2 += __ldcg(cp + 1);
                t.F2 += __ldcg(cp + 2);
                t.M2 = fmaxf(t.M2, __ldcg(cp + 3));
                t.A = fmaxf(t.A, __ldcg(cp + 4));
            }
            t = warp_reduce(t);
            if (threadIdx.x == 0) {
                mix_step(s, q, t);
                sh.coef = coef_of(s, need_anchor(s, q, t));
            }
        }
        __syncthreads();
        cur = nxt;
        if (sh.coef.anchor) {
            /* X += u (FP64), u = 0, then the FP64 anchor */
            for (int pp = blockIdx.x * NT + threadIdx.x; pp < tl.n_pos; pp += G * NT) {
                const int i = tl.node_of_pos[pp];
                if (i < 0) continue;
                const float4 w = tl.u[cur][pp];
                double2 x = d.x[i];
                x.x = x.x + ((double)w.x + (double)w.z);
                x.y = x.y + ((double)w.y + (double)w.w);
                d.x[i] = x;
                tl.u[cur][pp] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (!tile_barrier(tl, st, G, ++epoch, budget_ns, 23)) return;
            tile_anchor_eval(d, tl, cur, sh.dslots, tF2, tM2);
            if (threadIdx.x == 0) {
                tl.dpart[2 * blockIdx.x] = tF2;
                tl.dpart[2 * blockIdx.x + 1] = tM2;
            }
            if (!tile_barrier(tl, st, G, ++epoch, budget_ns, 24)) return;
            if (threadIdx.x == 0) {
                double F2, M2;
                tile_anchor_totals(tl, G, F2, M2);
                mix_certify(s, p, d.sqrt_dof, F2, M2);
                sh.coef = coef_of(s, 0);
            }
            __syncthreads();
            /* every CTA reads dpart before any CTA's next anchor rewrites
             * it: at least one step barrier lies between two anchors */
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) mix_report(st, s);
}

/* ------------------------------------------------------------------ */
/* Host side: layout and launch                                         */
/* ------------------------------------------------------------------ */

size_t tile_smem(const NetTile &tl) {
    return tile_smem_bytes(tl.max_ro, tl.max_nodes, tl.max_own, tl.max_bonds, tl.max_tris);
}

/* The kernel instantiation for `threads` per CTA (512, 768 or 256). */
static const void *tile_kernel(int threads) {
    if (threads == 256) return (const void *)k_fire_tile_mixed<256, 2>;
    if (threads == 768) return (const void *)k_fire_tile_mixed<768, 1>;
    return (const void *)k_fire_tile_mixed<512, 1>;
}

/* CTAs of the cooperative launch: co-resident CTAs per SM times SMs (0 when
 * the kernel cannot launch with this shared memory). */
int tile_grid_ctas(size_t smem, int threads) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    const void *k = tile_kernel(threads);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem) != cudaSuccess) return 0;
    return per_sm * sms;
}

cudaError_t launch_mixed_tile(const NetDev &d, const NetTile &tl, const FireParamsDev &p, int ctas, int threads,
                              unsigned long long budget_ns, cudaStream_t stream) {
    const void *k = tile_kernel(threads);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tile_smem(tl));
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(tl.bar, 0, sizeof(unsigned long long), stream)) != cudaSuccess) return e;
    NetDev dd = d;
    NetTile tt = tl;
    FireParamsDev pp = p;
    unsigned long long bb = budget_ns;
    void *args[] = {&dd, &tt, &pp, &bb};
    return launch_cooperative(k, ctas, threads, args, tile_smem(tl), stream);
}

/* Spatial tiles of one network (see NetTile): at most about target_nodes
 * nodes per tile, the tile count a multiple of `ctas`, equal-count cells in
 * strips of the box [0, width) x [miny, maxy] with the box's aspect ratio.
 * Returns NR_OK with the layout in `out` (host arrays), or NR_ERR_CAPACITY
 * when a tile exceeds the 16-bit local encoding. */
int build_tile_layout(const nr_host_network &h, const Incidence &inc, const unsigned char *fcodes, bool use_bonds,
                      bool use_triples, int ctas, int target_nodes, TileHost &out) {
    const int n = h.n_points, ne = h.n_edges(), nt = h.n_triples();
    const double W = h.offset, H = std::max(h.maxy - h.miny, 1e-300);
    if (n <= 0 || !(W > 0) || ctas < 1) return NR_ERR_INVALID;
    const long per = (long)ctas * target_nodes;
    const long want = (long)ctas * std::max(1L, (n + per - 1) / per);
    const int ny = (int)std::min(want, std::max(1L, std::lround(std::sqrt((double)want * H / W))));
    /* equal-count cells: ny strips of consecutive y, strip s cut into the
     * cells [want s / ny, want (s + 1) / ny) of consecutive x (periodic x
     * folded into [0, W)), each strip holding nodes in proportion to its
     * cells: exactly `want` cells (a multiple of ctas), each owning n / want
     * nodes however unevenly the nodes are spread (fibre networks), so no
     * tile's record is much larger than the mean and every CTA takes the
     * same number of tiles */
    const long ncells = want;
    std::vector<int> cell(n), count((size_t)ncells, 0), idx(n);
    std::vector<double> xs(n);
    for (int i = 0; i < n; ++i) {
        idx[i] = i;
        xs[i] = h.points[2 * i] - W * std::floor(h.points[2 * i] / W);
    }
    std::sort(idx.begin(), idx.end(), [&](int a, int b) {
        const double ya = h.points[2 * a + 1], yb = h.points[2 * b + 1];
        return ya < yb || (ya == yb && a < b);
    });
    for (int sy = 0; sy < ny; ++sy) {
        const long c0 = ncells * sy / ny, c1 = ncells * (sy + 1) / ny;
        const long lo = (long)n * c0 / ncells, hi = (long)n * c1 / ncells;
        std::sort(idx.begin() + lo, idx.begin() + hi,
                  [&](int a, int b) { return xs[a] < xs[b] || (xs[a] == xs[b] && a < b); });
        for (long k = lo; k < hi; ++k) {
            const long c = c0 + (k - lo) * (c1 - c0) / std::max(1L, hi - lo);
            cell[idx[k]] = (int)c;
            count[c]++;
        }
    }
    std::vector<int> tile_of_cell((size_t)ncells, -1);
    int T = 0;
    for (long c = 0; c < ncells; ++c)
        if (count[c] > 0) tile_of_cell[c] = T++;
    std::vector<std::vector<int>> own(T);
    for (int i = 0; i < n; ++i) own[tile_of_cell[cell[i]]].push_back(i); /* ascending */
    /* within a tile, own nodes by their numbers of triple and bond entries:
     * the lanes of a warp gather (nearly) equally long incidence lists */
    auto entries = [&](int i, bool tri) {
        if (tri) return use_triples ? inc.tptr[i + 1] - inc.tptr[i] : 0;
        return use_bonds ? inc.bptr[i + 1] - inc.bptr[i] : 0;
    };
    for (std::vector<int> &o : own)
        std::stable_sort(o.begin(), o.end(), [&](int a, int b) {
            const int ta = entries(a, true), tb = entries(b, true);
            return ta != tb ? ta > tb : entries(a, false) > entries(b, false);
        });
    out = TileHost();
    out.n_tiles = T;
    /* tile-order positions: each tile's own range starts on a multiple of 16 */
    std::vector<int> pos_of(n), own_pos(T);
    int P = 0;
    for (int t = 0; t < T; ++t) {
        own_pos[t] = P;
        for (size_t k = 0; k < own[t].size(); ++k) pos_of[own[t][k]] = P + (int)k;
        P += (int)((own[t].size() + 15) / 16 * 16);
    }
    out.n_pos = P;
    out.node_of_pos.assign(P, -1);
    for (int i = 0; i < n; ++i) out.node_of_pos[pos_of[i]] = i;
    std::vector<int> loc(n, -1), bslot(use_bonds ? ne : 0, -1), tslot(use_triples ? nt : 0, -1);
    std::vector<int> bl, tlist, halo;
    std::vector<unsigned short> iptr, ibe, incv;
    for (int t = 0; t < T; ++t) {
        const std::vector<int> &o = own[t];
        for (size_t k = 0; k < o.size(); ++k) loc[o[k]] = (int)k;
        bl.clear();
        tlist.clear();
        halo.clear();
        for (int i : o) {
            if (use_bonds)
                for (int e = inc.bptr[i]; e < inc.bptr[i + 1]; ++e) bl.push_back(inc.bent[e] >> 1);
            if (use_triples)
                for (int e = inc.tptr[i]; e < inc.tptr[i + 1]; ++e) tlist.push_back(inc.tent[e] >> 2);
        }
        std::sort(bl.begin(), bl.end());
        bl.erase(std::unique(bl.begin(), bl.end()), bl.end());
        std::sort(tlist.begin(), tlist.end());
        tlist.erase(std::unique(tlist.begin(), tlist.end()), tlist.end());
        auto touch = [&](int v) {
            if (loc[v] == -1) {
                loc[v] = -2; /* halo, numbered below */
                halo.push_back(v);
            }
        };
        for (int b : bl) {
            touch(h.edge_ij[2 * b]);
            touch(h.edge_ij[2 * b + 1]);
        }
        for (int qq : tlist)
            for (int r = 0; r < 3; ++r) touch(h.tri_hjk[3 * qq + r]);
        std::sort(halo.begin(), halo.end());
        for (size_t k = 0; k < halo.size(); ++k) loc[halo[k]] = (int)(o.size() + k);
        auto reset = [&]() {
            for (int v : o) loc[v] = -1;
            for (int v : halo) loc[v] = -1;
            for (int b : bl) bslot[b] = -1;
            for (int qq : tlist) tslot[qq] = -1;
        };
        const size_t nn = o.size() + halo.size();
        if (nn > 0xffff || bl.size() >= 0x4000 || tlist.size() >= 0x2000) {
            reset();
            return NR_ERR_CAPACITY;
        }
        for (size_t k = 0; k < bl.size(); ++k) bslot[bl[k]] = (int)k;
        for (size_t k = 0; k < tlist.size(); ++k) tslot[tlist[k]] = (int)k;
        /* incidence of the own nodes, canonical order: bonds, then triples */
        iptr.clear();
        ibe.clear();
        incv.clear();
        for (int i : o) {
            iptr.push_back((unsigned short)incv.size());
            if (use_bonds)
                for (int e = inc.bptr[i]; e < inc.bptr[i + 1]; ++e)
                    incv.push_back((unsigned short)((bslot[inc.bent[e] >> 1] << 1) | (inc.bent[e] & 1)));
            ibe.push_back((unsigned short)incv.size());
            if (use_triples)
                for (int e = inc.tptr[i]; e < inc.tptr[i + 1]; ++e)
                    incv.push_back((unsigned short)(0x8000 | (tslot[inc.tent[e] >> 2] << 2) | (inc.tent[e] & 3)));
            if (incv.size() > 0xffff) {
                reset();
                return NR_ERR_CAPACITY;
            }
        }
        iptr.push_back((unsigned short)incv.size());
        TileDesc td;
        td.ro_off = (long long)out.ro.size();
        td.own_pos = own_pos[t];
        td.no = (int)o.size();
        td.nh = (int)halo.size();
        td.nb = (int)bl.size();
        td.nt = (int)tlist.size();
        td.ni = (int)incv.size();
        td.bond_off = (int)out.bid.size();
        td.tri_off = (int)out.tid.size();
        td.pad = 0;
        const TileSegs g = tile_segs(td.nb, td.nt, td.no, td.ni, td.nh);
        out.ro.resize(out.ro.size() + g.total, 0);
        unsigned char *rec = out.ro.data() + td.ro_off;
        for (size_t k = 0; k < bl.size(); ++k) {
            const int b = bl[k];
            const unsigned r = (unsigned)loc[h.edge_ij[2 * b]] | ((unsigned)loc[h.edge_ij[2 * b + 1]] << 16);
            memcpy(rec + g.bref + 4 * k, &r, 4);
            out.bid.push_back(b);
        }
        for (size_t k = 0; k < tlist.size(); ++k) {
            const int qq = tlist[k];
            const uint2 r = make_uint2((unsigned)loc[h.tri_hjk[3 * qq]] | ((unsigned)loc[h.tri_hjk[3 * qq + 1]] << 16),
                                       (unsigned)loc[h.tri_hjk[3 * qq + 2]]);
            memcpy(rec + g.tref + 8 * k, &r, 8);
            out.tid.push_back(qq);
        }
        memcpy(rec + g.iptr, iptr.data(), 2 * iptr.size());
        if (!ibe.empty()) memcpy(rec + g.ibe, ibe.data(), 2 * ibe.size());
        if (!incv.empty()) memcpy(rec + g.inc, incv.data(), 2 * incv.size());
        for (size_t k = 0; k < o.size(); ++k) rec[g.fcode + k] = fcodes[o[k]];
        for (size_t k = 0; k < halo.size(); ++k) {
            const int pp = pos_of[halo[k]];
            memcpy(rec + g.halo + 4 * k, &pp, 4);
        }
        out.desc.push_back(td);
        out.max_nodes = std::max(out.max_nodes, (int)nn);
        out.max_own = std::max(out.max_own, td.no);
        out.max_bonds = std::max(out.max_bonds, td.nb);
        out.max_tris = std::max(out.max_tris, td.nt);
        out.max_ro = std::max(out.max_ro, g.total);
        reset();
    }
    out.max_nodes = std::max(out.max_nodes, 1);
    out.max_own = std::max(out.max_own, 1);
    out.max_bonds = std::max(out.max_bonds, 1);
    out.max_tris = std::max(out.max_tris, 1);
    out.max_ro = std::max(out.max_ro, 16u);
    return NR_OK;
}

}  // namespace nr

extern "C" int nr_tile_layout_check(const nr_host_network *h, int ctas, int target_nodes, long long stats[6]) {
    using namespace nr;
    if (!h || !stats || ctas < 1 || target_nodes < 1) return NR_ERR_INVALID;
    for (int k = 0; k < 6; ++k) stats[k] = 0;
    const int n = h->n_points, ne = h->n_edges(), nt = h->n_triples();
    Incidence inc;
    build_incidence(n, h->edge_ij.data(), ne, h->tri_hjk.data(), nt, true, true, inc);
    std::vector<unsigned char> fc(n);
    nr_host_network_fcodes(h, fc.data());
    TileHost th;
    const int rc = build_tile_layout(*h, inc, fc.data(), true, true, ctas, target_nodes, th);
    if (rc != NR_OK) return rc;
    long long bad = 0, halo_total = 0;
    std::vector<int> owned(n, 0);
    for (int t = 0; t < th.n_tiles; ++t) {
        const TileDesc &td = th.desc[t];
        const TileSegs g = tile_segs(td.nb, td.nt, td.no, td.ni, td.nh);
        if (td.ro_off % 16 || g.total % 16 || td.ro_off + (long long)g.total > (long long)th.ro.size() ||
            g.total > th.max_ro) {
            ++bad;
            continue;
        }
        if (td.own_pos % 16 || td.own_pos + td.no > th.n_pos || td.no + td.nh > th.max_nodes ||
            td.nb > th.max_bonds || td.nt > th.max_tris || td.no > th.max_own)
            ++bad;
        const unsigned char *rec = th.ro.data() + td.ro_off;
        const int nn = td.no + td.nh;
        for (int k = 0; k < td.no; ++k) {
            const int i = th.node_of_pos[td.own_pos + k];
            if (i < 0 || i >= n) {
                ++bad;
                continue;
            }
            owned[i]++;
            if (rec[g.fcode + k] != fc[i]) ++bad;
        }
        for (int k = 0; k < td.nb; ++k) {
            unsigned r;
            memcpy(&r, rec + g.bref + 4 * k, 4);
            if ((int)(r & 0xffffu) >= nn || (int)(r >> 16) >= nn) ++bad;
            const int b = th.bid[td.bond_off + k];
            if (b < 0 || b >= ne) ++bad;
        }
        for (int k = 0; k < td.nt; ++k) {
            unsigned r[2];
            memcpy(r, rec + g.tref + 8 * k, 8);
            if ((int)(r[0] & 0xffffu) >= nn || (int)(r[0] >> 16) >= nn || (int)r[1] >= nn) ++bad;
            const int q = th.tid[td.tri_off + k];
            if (q < 0 || q >= nt) ++bad;
        }
        for (int k = 0; k < td.nh; ++k) {
            int pp;
            memcpy(&pp, rec + g.halo + 4 * k, 4);
            if (pp < 0 || pp >= th.n_pos || th.node_of_pos[pp] < 0) ++bad;
        }
        for (int k = 0; k < td.no; ++k) {
            unsigned short a, b, e;
            memcpy(&a, rec + g.iptr + 2 * k, 2);
            memcpy(&e, rec + g.iptr + 2 * k + 2, 2);
            memcpy(&b, rec + g.ibe + 2 * k, 2);
            if (!(a <= b && b <= e && e <= td.ni)) {
                ++bad;
                continue;
            }
            for (int x = a; x < e; ++x) {
                unsigned short c;
                memcpy(&c, rec + g.inc + 2 * x, 2);
                const bool tri = (c & 0x8000u) != 0;
                if (tri != (x >= b)) ++bad;
                if (!tri && (c >> 1) >= (unsigned)td.nb) ++bad;
                if (tri && (((c & 0x7fffu) >> 2) >= (unsigned)td.nt || (c & 3u) > 2u)) ++bad;
            }
        }
        halo_total += td.nh;
    }
    for (int i = 0; i < n; ++i)
        if (owned[i] != 1) ++bad;
    stats[0] = th.n_tiles;
    stats[1] = th.n_pos;
    stats[2] = th.max_nodes;
    stats[3] = th.max_ro;
    stats[4] = halo_total;
    stats[5] = bad;
    return NR_OK;
}

