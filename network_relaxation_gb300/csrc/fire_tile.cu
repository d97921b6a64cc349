/*
 * Mixed-precision FIRE for one large network over the whole GPU, in spatial
 * tiles, with ONE grid barrier per FIRE step.
 *
 * The cooperative grid kernel of fire_mixed.cu runs a step as four passes
 * separated by grid barriers (drift, item pass writing every bond's and
 * triple's FP32 force change to global memory, gather reading them back,
 * reduction by the last CTA) and is bound by the latency of those passes and
 * barriers.  Here a CTA takes whole tiles (NetTile, nr_device.cuh: a spatial
 * block of nodes, its halo and every item touching it, stored tile-major)
 * and does the whole step of a tile on chip:
 *   1. load u, v, F of the tile's own and halo nodes (from the step's input
 *      copy of the double-buffered state) into shared memory;
 *   2. pass A (mixing, drift, half kick) for own AND halo nodes: the halo's
 *      drift is recomputed from the same inputs with the same operations as
 *      its owner's, so it has the same bits, and no barrier is needed
 *      between the drift and the items;
 *   3. the item pass: the FP32 force change of every bond and triple of the
 *      tile into shared memory (boundary items are evaluated by each tile
 *      they touch, identically);
 *   4. the gather of the tile's own nodes in the canonical incidence order,
 *      half kick, writes of u, v, F to the step's output copy, and the
 *      step's partial sums.
 * Then one grid barrier; every CTA combines the CTAs' partial sums in CTA
 * order itself and advances an identical copy of the FIRE scalars.  The
 * arithmetic (double-float u, bond_dforce, tri_dforce, FP32 FIRE step, FP64
 * anchors and certification) is mixed_common.cuh's; per node the force is
 * the same sum in the same order as in the other mixed kernels.  Anchors
 * (rare) take two more barriers: X += u, then the FP64 force and the tile
 * items' FP32 anchor records.
 *
 * Compiled with --fmad=false; FP32 expressions use explicit fmaf().
 */
#include <algorithm>
#include <cmath>
#include <vector>

#include "mixed_common.cuh"
#include "nr_internal.h"

namespace nr {

/* ----- grid barrier: a monotonic counter, every CTA waits for all ----- */

/* Arrives at barrier number `epoch` (1, 2, ...) of the launch and waits
 * until all G CTAs have; false when the wait exceeded budget_ns or another
 * CTA gave up (st->abort_flag), every thread of the CTA sees the same
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

/* Dynamic shared memory of a CTA: one tile's state and item results. */
struct TileSmem {
    float4 *u, *tdf;
    float2 *v, *bdf;
};
__host__ __device__ inline size_t tile_smem_bytes(int max_nodes, int max_bonds, int max_tris) {
    return 16 * (size_t)max_nodes + 16 * (size_t)max_tris + 8 * (size_t)max_nodes + 8 * (size_t)max_bonds;
}

/* FP64 anchor evaluation: X += u was done; every node's canonical FP64
 * force (d.f), its double-float copy (fa) and F = fa_hi in the current state
 * copy; the FP32 anchor records of the CTA's tiles' items.  Returns the CTA
 * partials of |F|^2 (sum) and max |F|^2 in thread 0. */
static __device__ __noinline__ void tile_anchor_eval(const NetDev &d, const NetTile &tl, int cur, double *dslots,
                                                     double &tF2, double &tM2) {
    const double W = d.width;
    double F2 = 0.0, M2 = 0.0;
    const int G = gridDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += G * blockDim.x) {
        double fx, fy;
        node_force_fp64_own<false>(d, i, fx, fy);
        d.f[i] = make_double2(fx, fy);
        const float hx = (float)fx, hy = (float)fy;
        d.fa_hi[i] = make_float2(hx, hy);
        d.fa_lo[i] = make_float2((float)(fx - (double)hx), (float)(fy - (double)hy));
        tl.f[cur][i] = make_float2(hx, hy);
        const double t = dot2(fx, fy, fx, fy);
        F2 += t;
        M2 = fmax(M2, t);
    }
    for (int t = blockIdx.x; t < tl.n_tiles; t += G) {
        if (d.use_bonds)
            for (int k = tl.bond_off[t] + threadIdx.x; k < tl.bond_off[t + 1]; k += blockDim.x) {
                const int b = tl.bid[k];
                const int4 r = d.bond[b];
                const double2 p1 = d.x[r.x], p2 = d.x[r.y];
                const double rx = (p2.x + wrap_shift(r.z, W)) - p1.x, ry = p2.y - p1.y;
                const double kk = d.bond_k ? d.bond_k[b] : d.ks;
                const float hx = (float)rx, hy = (float)ry;
                tl.mb[k] = make_float4(hx, hy, (float)(rx - (double)hx), (float)(ry - (double)hy));
                tl.sk[k] = make_float2((float)(sqrt(fma(rx, rx, ry * ry)) - d.bond_l0[b]), (float)kk);
            }
        if (d.use_triples)
            for (int k = tl.tri_off[t] + threadIdx.x; k < tl.tri_off[t + 1]; k += blockDim.x) {
                const int tt = tl.tid[k];
                const int4 r = d.tri[tt];
                const double2 ph = d.x[r.x], pj = d.x[r.y], pk = d.x[r.z];
                const int wj = (signed char)(r.w & 0xff), wk = (signed char)((r.w >> 8) & 0xff);
                const double ax = (pj.x + wrap_shift(wj, W)) - ph.x, ay = pj.y - ph.y;
                const double bx = (pk.x + wrap_shift(wk, W)) - ph.x, by = pk.y - ph.y;
                const double kb = d.tri_kb ? d.tri_kb[tt] : d.kb;
                const double phi0 = d.tri_phi0 ? d.tri_phi0[tt] : 0.0;
                tl.arms[k] = make_float4((float)ax, (float)ay, (float)bx, (float)by);
                tl.pk[k] = make_float2((float)bend_dtheta(ax, ay, bx, by, phi0), (float)kb);
            }
    }
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

/* Pass A of one node held in shared memory (mixed_pass_a's operations). */
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

template <int NT>
__global__ void __launch_bounds__(NT, 2)
    k_fire_tile_mixed(NetDev d, NetTile tl, FireParamsDev p, unsigned long long budget_ns) {
    extern __shared__ float4 s_dyn[];
    __shared__ MixShared sh;
    unsigned char *dyn = reinterpret_cast<unsigned char *>(s_dyn);
    TileSmem sm;
    sm.u = reinterpret_cast<float4 *>(dyn);
    sm.tdf = sm.u + tl.max_nodes;
    sm.v = reinterpret_cast<float2 *>(sm.tdf + tl.max_tris);
    sm.bdf = sm.v + tl.max_nodes;
    const unsigned G = gridDim.x;
    FireState *st = d.st;
    unsigned long long epoch = 0;
    /* FIRE scalars, advanced by thread 0 of every CTA (identical copies);
     * kept in shared memory, out of the step loop's registers */
    __shared__ MixScal s;
    __shared__ MixParams q;
    if (threadIdx.x == 0) q = mix_params(p, d.sqrt_dof);
    int cur = 0;
    for (int i = blockIdx.x * NT + threadIdx.x; i < d.n; i += G * NT) {
        tl.u[0][i] = make_float4(0.f, 0.f, 0.f, 0.f);
        tl.v[0][i] = make_float2(0.f, 0.f);
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
    for (;;) {
        const Coef &c = sh.coef;
        if (c.done) {
            /* the last pass A: mixing of v only (u is 0 after the certifying
             * anchor); the FP64 velocities out */
            for (int i = blockIdx.x * NT + threadIdx.x; i < d.n; i += G * NT) {
                float4 w = tl.u[cur][i];
                float2 v = tl.v[cur][i];
                tile_pass_a(c, w, v, tl.f[cur][i]);
                d.v[i] = make_double2((double)v.x, (double)v.y);
            }
            break;
        }
        const int nxt = cur ^ 1;
        float P = 0.f, V2 = 0.f, Fs = 0.f, M2f = 0.f, A = 0.f;
        for (int t = blockIdx.x; t < tl.n_tiles; t += G) {
            const int n0 = tl.node_off[t], no = tl.n_own[t], nn = no + tl.n_halo[t];
            const int b0 = tl.bond_off[t], nb = tl.bond_off[t + 1] - b0;
            const int t0 = tl.tri_off[t], ntr = tl.tri_off[t + 1] - t0;
            /* 1 + 2: state of own and halo nodes, then their pass A */
            for (int k = threadIdx.x; k < nn; k += NT) {
                const int i = __ldg(tl.node + n0 + k);
                float4 w = tl.u[cur][i];
                float2 v = tl.v[cur][i];
                const float2 F = tl.f[cur][i];
                tile_pass_a(c, w, v, F);
                sm.u[k] = w;
                sm.v[k] = v;
            }
            __syncthreads();
            /* 3: item pass into shared memory */
            if (d.use_bonds)
                for (int k = threadIdx.x; k < nb; k += NT) {
                    const unsigned r = __ldg(tl.bref + b0 + k);
                    const float4 ra = tl.mb[b0 + k];
                    const float2 sk = tl.sk[b0 + k];
                    const float4 ui = sm.u[r & 0xffffu], uj = sm.u[r >> 16];
                    float2 dh, dlo;
                    u_diff2(make_float2(uj.x, uj.y), make_float2(uj.z, uj.w), make_float2(ui.x, ui.y),
                            make_float2(ui.z, ui.w), dh, dlo);
                    sm.bdf[k] = bond_dforce(ra, sk, dh, dlo);
                }
            if (d.use_triples)
                for (int k = threadIdx.x; k < ntr; k += NT) {
                    const uint2 r = __ldg(tl.tref + t0 + k);
                    const float4 arms = tl.arms[t0 + k];
                    const float2 pk = tl.pk[t0 + k];
                    const float4 uh = sm.u[r.x & 0xffffu], uj = sm.u[r.x >> 16], uk = sm.u[r.y];
                    const float2 hh = make_float2(uh.x, uh.y), hl = make_float2(uh.z, uh.w);
                    float2 dFj, dFk;
                    tri_dforce(arms, pk, u_diff(make_float2(uj.x, uj.y), make_float2(uj.z, uj.w), hh, hl),
                               u_diff(make_float2(uk.x, uk.y), make_float2(uk.z, uk.w), hh, hl), dFj, dFk);
                    sm.tdf[k] = make_float4(dFj.x, dFj.y, dFk.x, dFk.y);
                }
            __syncthreads();
            /* 4: gather of the own nodes, half kick, the next step's state */
            const unsigned short *ip = tl.iptr + tl.own_off[t] + t;
            const unsigned short *inc = tl.inc + tl.inc_off[t];
            for (int k = threadIdx.x; k < no; k += NT) {
                const int i = __ldg(tl.node + n0 + k);
                const unsigned fc = __ldg(d.fcode + i);
                const int e0 = __ldg(ip + k), e1 = __ldg(ip + k + 1);
                const float2 ah = d.fa_hi[i], al = d.fa_lo[i];
                float2 F = make_float2(0.f, 0.f);
                if (fc != 0) {
                    float2 dF = make_float2(0.f, 0.f);
                    float mag = 0.f;
                    for (int e = e0; e < e1; ++e) {
                        const unsigned code = __ldg(inc + e);
                        if (!(code & 0x8000u)) {
                            float2 df = sm.bdf[code >> 1];
                            if (code & 1) df = make_float2(-df.x, -df.y);
                            dF.x += df.x;
                            dF.y += df.y;
                            mag += fabsf(df.x) + fabsf(df.y);
                        } else {
                            const int role = code & 3;
                            const float4 qv = sm.tdf[(code & 0x7fffu) >> 2];
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
                float2 v = sm.v[k];
                v.x = fmaf(c.dtm, F.x, v.x);
                v.y = fmaf(c.dtm, F.y, v.y);
                tl.u[nxt][i] = sm.u[k];
                tl.v[nxt][i] = v;
                tl.f[nxt][i] = F;
                P += fmaf(v.x, F.x, v.y * F.y);
                V2 += fmaf(v.x, v.x, v.y * v.y);
                const float f2 = fmaf(F.x, F.x, F.y * F.y);
                Fs += f2;
                M2f = fmaxf(M2f, f2);
            }
            __syncthreads();
        }
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
            for (int k = threadIdx.x; k < (int)G; k += 32) {
                const float *cp = tl.cpart + 5 * ((size_t)cur * G + k);
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
            for (int i = blockIdx.x * NT + threadIdx.x; i < d.n; i += G * NT) {
                const float4 w = tl.u[cur][i];
                double2 x = d.x[i];
                x.x = x.x + ((double)w.x + (double)w.z);
                x.y = x.y + ((double)w.y + (double)w.w);
                d.x[i] = x;
                tl.u[cur][i] = make_float4(0.f, 0.f, 0.f, 0.f);
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

constexpr int kTileThreads = 512;

/* CTAs of the cooperative launch: co-resident CTAs per SM times SMs
 * (0 when the kernel cannot launch with this shared memory). */
int tile_grid_ctas(size_t smem) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaFuncSetAttribute(k_fire_tile_mixed<kTileThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fire_tile_mixed<kTileThreads>, kTileThreads, smem) !=
        cudaSuccess)
        return 0;
    return per_sm * sms;
}

size_t tile_smem(const NetTile &tl) { return tile_smem_bytes(tl.max_nodes, tl.max_bonds, tl.max_tris); }

cudaError_t launch_mixed_tile(const NetDev &d, const NetTile &tl, const FireParamsDev &p, int ctas,
                              unsigned long long budget_ns, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(tl.bar, 0, sizeof(unsigned long long), stream);
    if (e != cudaSuccess) return e;
    NetDev dd = d;
    NetTile tt = tl;
    FireParamsDev pp = p;
    unsigned long long bb = budget_ns;
    void *args[] = {&dd, &tt, &pp, &bb};
    return launch_cooperative((const void *)k_fire_tile_mixed<kTileThreads>, ctas, kTileThreads, args, tile_smem(tl),
                              stream);
}

/* Spatial tiles of one network (see NetTile): about target_nodes nodes per
 * tile, the tile count a multiple of `ctas` (each CTA takes the same number
 * of tiles), cells of the box [0, width) x [miny, maxy] with the box's
 * aspect ratio.  Returns NR_OK with the layout in `out` (host arrays),
 * or NR_ERR_CAPACITY when a tile exceeds the 16-bit local encoding. */
int build_tile_layout(const nr_host_network &h, const Incidence &inc, bool use_bonds, bool use_triples, int ctas,
                      int target_nodes, TileHost &out) {
    const int n = h.n_points, ne = h.n_edges(), nt = h.n_triples();
    const double W = h.offset, y0 = h.miny, H = std::max(h.maxy - h.miny, 1e-300);
    if (n <= 0 || !(W > 0) || ctas < 1) return NR_ERR_INVALID;
    const long per = (long)ctas * target_nodes;
    const long want = (long)ctas * std::max(1L, (n + per - 1) / per);
    int ny = std::max(1, (int)std::lround(std::sqrt((double)want * H / W)));
    int nx = std::max(1, (int)((want + ny - 1) / ny));
    std::vector<int> cell(n), count((size_t)nx * ny + 1, 0);
    for (int i = 0; i < n; ++i) {
        double x = h.points[2 * i], y = h.points[2 * i + 1];
        x -= W * std::floor(x / W);
        int cx = std::min(nx - 1, std::max(0, (int)(x / W * nx)));
        int cy = std::min(ny - 1, std::max(0, (int)((y - y0) / H * ny)));
        cell[i] = cy * nx + cx;
        count[cell[i] + 1]++;
    }
    /* compact the non-empty cells into tiles, cells in row order */
    std::vector<int> tile_of_cell((size_t)nx * ny, -1);
    int T = 0;
    for (int cidx = 0; cidx < nx * ny; ++cidx)
        if (count[cidx + 1] > 0) tile_of_cell[cidx] = T++;
    std::vector<std::vector<int>> own(T);
    for (int i = 0; i < n; ++i) own[tile_of_cell[cell[i]]].push_back(i); /* ascending */
    out = TileHost();
    out.n_tiles = T;
    out.node_off.push_back(0);
    out.own_off.push_back(0);
    out.bond_off.push_back(0);
    out.tri_off.push_back(0);
    out.inc_off.push_back(0);
    std::vector<int> loc(n, -1), bslot(use_bonds ? ne : 0, -1), tslot(use_triples ? nt : 0, -1);
    std::vector<int> bl, tlist, halo;
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
            if (loc[v] < 0) {
                loc[v] = -2; /* halo, numbered below */
                halo.push_back(v);
            }
        };
        for (int b : bl) {
            touch(h.edge_ij[2 * b]);
            touch(h.edge_ij[2 * b + 1]);
        }
        for (int q : tlist)
            for (int r = 0; r < 3; ++r) touch(h.tri_hjk[3 * q + r]);
        std::sort(halo.begin(), halo.end());
        for (size_t k = 0; k < halo.size(); ++k) loc[halo[k]] = (int)(o.size() + k);
        const size_t nn = o.size() + halo.size();
        if (nn > 0xffff || bl.size() >= 0x4000 || tlist.size() >= 0x2000) {
            for (int v : o) loc[v] = -1;
            for (int v : halo) loc[v] = -1;
            return NR_ERR_CAPACITY;
        }
        out.n_own.push_back((int)o.size());
        out.n_halo.push_back((int)halo.size());
        out.node.insert(out.node.end(), o.begin(), o.end());
        out.node.insert(out.node.end(), halo.begin(), halo.end());
        for (size_t k = 0; k < bl.size(); ++k) {
            const int b = bl[k];
            bslot[b] = (int)k;
            out.bref.push_back((unsigned)loc[h.edge_ij[2 * b]] | ((unsigned)loc[h.edge_ij[2 * b + 1]] << 16));
            out.bid.push_back(b);
        }
        for (size_t k = 0; k < tlist.size(); ++k) {
            const int q = tlist[k];
            tslot[q] = (int)k;
            out.tref.push_back(make_uint2((unsigned)loc[h.tri_hjk[3 * q]] | ((unsigned)loc[h.tri_hjk[3 * q + 1]] << 16),
                                          (unsigned)loc[h.tri_hjk[3 * q + 2]]));
            out.tid.push_back(q);
        }
        /* incidence of the own nodes, canonical order: bonds, then triples */
        const size_t ibase = out.inc.size();
        for (int i : o) {
            out.iptr.push_back((unsigned short)(out.inc.size() - ibase));
            if (use_bonds)
                for (int e = inc.bptr[i]; e < inc.bptr[i + 1]; ++e) {
                    const int b = inc.bent[e] >> 1, role = inc.bent[e] & 1;
                    out.inc.push_back((unsigned short)((bslot[b] << 1) | role));
                }
            if (use_triples)
                for (int e = inc.tptr[i]; e < inc.tptr[i + 1]; ++e) {
                    const int q = inc.tent[e] >> 2, role = inc.tent[e] & 3;
                    out.inc.push_back((unsigned short)(0x8000 | (tslot[q] << 2) | role));
                }
        }
        if (out.inc.size() - ibase > 0xffff) return NR_ERR_CAPACITY;
        out.iptr.push_back((unsigned short)(out.inc.size() - ibase));
        out.max_nodes = std::max(out.max_nodes, (int)nn);
        out.max_bonds = std::max(out.max_bonds, (int)bl.size());
        out.max_tris = std::max(out.max_tris, (int)tlist.size());
        out.node_off.push_back((int)out.node.size());
        out.own_off.push_back(out.own_off.back() + (int)o.size());
        out.bond_off.push_back((int)out.bid.size());
        out.tri_off.push_back((int)out.tid.size());
        out.inc_off.push_back((int)out.inc.size());
        for (int v : o) loc[v] = -1;
        for (int v : halo) loc[v] = -1;
        for (int b : bl) bslot[b] = -1;
        for (int q : tlist) tslot[q] = -1;
    }
    out.max_nodes = std::max(out.max_nodes, 1);
    out.max_bonds = std::max(out.max_bonds, 1);
    out.max_tris = std::max(out.max_tris, 1);
    return NR_OK;
}

}  // namespace nr
