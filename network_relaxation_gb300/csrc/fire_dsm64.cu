/*
 * Plain FP64 FIRE (the run_fire_md drop-in's arithmetic, bit-identical to
 * the oracle) on one thread-block cluster per network with the step's state
 * in distributed shared memory.
 *
 * On GB300 a small network's FP64 step is bound by latency, not by the FP64
 * pipe: in the grid kernel by its software grid barriers, in the L2 cluster
 * kernel (k_fire_cluster) by chains of dependent L2 loads (incidence ->
 * item force, bond -> positions) and the reduction's L2 reads.  Here every
 * value a step writes and reads back is on chip:
 *   per node (owner CTA)   x, v, F (double2 each)
 *   per item (owner CTA)   the bond's force on its node i (double2), the
 *                          triple's forces on j and k (double4)
 *   per 32-node chunk      its partial sums of P, |v|^2, |F|^2, max |F|^2
 * A CTA reads other CTAs' positions (item pass), item forces (gather) and
 * chunk partials (reduction) with ld.shared::cluster after the hardware
 * cluster barrier that ends the producing pass.  The layout is NetDsm's
 * (nr_device.cuh), whose sub-blocks are whole 32-node chunks, so a CTA's
 * nodes are whole reduction units: every CTA computes the canonical totals
 * (the oracle's tree: chunk butterflies, trees of 8, per-lane tile
 * accumulation) from all chunks itself and advances an identical copy of
 * the FP64 FIRE scalars; three cluster barriers per step.  A thread's item
 * and node are the same every step, so their read-only data (node
 * references, rest length, stiffness, wraps, incidence range) is loaded
 * once per relaxation into registers.
 *
 * Compiled with --fmad=false: the same bits as the oracle.
 */
#include <cooperative_groups.h>

#include <algorithm>

#include "fire_common.cuh"
#include "fire_launch.h"

namespace nr {

namespace {

__device__ __forceinline__ unsigned cl_addr(const void *p, unsigned rank) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ double2 cl_ld2d(unsigned a) {
    double2 v;
    asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(a));
    return v;
}
__device__ __forceinline__ double cl_ld1d(unsigned a) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(a));
    return v;
}
__device__ __forceinline__ double4 cl_ld4d(unsigned a) {
    const double2 lo = cl_ld2d(a), hi = cl_ld2d(a + 16u);
    return make_double4(lo.x, lo.y, hi.x, hi.y);
}

}  // namespace

/* Per-CTA maxima of a launch: nodes, bond slots, triple slots. */
struct Dsm64Sizes {
    int bmax, emax, tmax;
};
struct Dsm64Layout {
    size_t x, v, f, bf, tf, part, total;
};
__host__ __device__ inline Dsm64Layout dsm64_layout(const Dsm64Sizes &z) {
    Dsm64Layout L;
    size_t o = 0;
    L.x = o;  o += 16 * (size_t)z.bmax;
    L.v = o;  o += 16 * (size_t)z.bmax;
    L.f = o;  o += 16 * (size_t)z.bmax;
    L.bf = o; o += 16 * (size_t)z.emax;
    L.tf = o; o += 32 * (size_t)z.tmax;
    L.part = o; o += 4 * 8 * (size_t)((z.bmax + kChunk - 1) / kChunk);
    L.total = o;
    return L;
}

constexpr int kDsm64Threads = 256;

__global__ void __launch_bounds__(kDsm64Threads, 1)
    k_fire_dsm64(const NetDev *nets, const NetDsm *dsms, int n_nets, FireParamsDev p, int *queue, const int *order,
                 Dsm64Sizes z) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    extern __shared__ double2 s_dyn64[];
    unsigned char *dyn = reinterpret_cast<unsigned char *>(s_dyn64);
    const Dsm64Layout L = dsm64_layout(z);
    double2 *s_x = reinterpret_cast<double2 *>(dyn + L.x);
    double2 *s_v = reinterpret_cast<double2 *>(dyn + L.v);
    double2 *s_f = reinterpret_cast<double2 *>(dyn + L.f);
    double2 *s_bf = reinterpret_cast<double2 *>(dyn + L.bf);
    double4 *s_tf = reinterpret_cast<double4 *>(dyn + L.tf);
    double *s_part = reinterpret_cast<double *>(dyn + L.part); /* [q * umax + local chunk] */
    const int umax = (z.bmax + kChunk - 1) / kChunk;
    __shared__ NetDev s_d;
    __shared__ NetDsm s_m;
    __shared__ Scal s_sc;
    __shared__ int s_slot;
    __shared__ double s_red[32];
    __shared__ unsigned s_ax[kDsmParts], s_abf[kDsmParts], s_atf[kDsmParts], s_apt[kDsmParts];
    const int rank = (int)cl.block_rank(), C = (int)cl.num_blocks();
    const int spr = kDsmParts / C, lg = __ffs(spr) - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if ((int)threadIdx.x < C) {
        s_ax[threadIdx.x] = cl_addr(s_x, threadIdx.x);
        s_abf[threadIdx.x] = cl_addr(s_bf, threadIdx.x);
        s_atf[threadIdx.x] = cl_addr(s_tf, threadIdx.x);
        s_apt[threadIdx.x] = cl_addr(s_part, threadIdx.x);
    }
    for (;;) {
        if (rank == 0 && threadIdx.x == 0) s_slot = atomicAdd(queue, 1);
        cl.sync();
        const int slot = *cl.map_shared_rank(&s_slot, 0);
        cl.sync(); /* every CTA read rank 0's slot before any may exit */
        if (slot >= n_nets) return;
        if (threadIdx.x == 0) {
            const int idx = order ? order[slot] : slot;
            s_d = nets[idx];
            s_m = dsms[idx];
        }
        __syncthreads();
        const NetDev &d = s_d;
        const NetDsm &m = s_m;
        const int bsub = m.bsub, per = spr * bsub; /* nodes of each CTA's range */
        const int n0 = rank * per, nloc = max(0, min(per, d.n - n0));
        const int b0 = m.bo[rank * spr], b1 = m.bo[(rank + 1) * spr];
        const int t0 = m.to[rank * spr], t1 = m.to[(rank + 1) * spr];
        const double W = d.width;
        const int n_units = d.n_tiles * 8;
        /* positions in */
        for (int li = threadIdx.x; li < nloc; li += blockDim.x) s_x[li] = d.x[n0 + li];
        /* the thread's first bond and triple, cached for the relaxation */
        const int nb = d.use_bonds ? b1 - b0 : 0, nt = d.use_triples ? t1 - t0 : 0;
        int cb_i = 0, cb_j = 0;
        double cb_w = 0.0, cb_l0 = 0.0, cb_k = 0.0;
        if ((int)threadIdx.x < nb) {
            const int2 r = __ldg(m.bref + b0 + threadIdx.x);
            const int b = __ldg(m.bidx + b0 + threadIdx.x);
            cb_i = r.x;
            cb_j = r.y;
            cb_w = wrap_shift(__ldg(&d.bond[b].z), W);
            cb_l0 = __ldg(d.bond_l0 + b);
            cb_k = d.bond_k ? __ldg(d.bond_k + b) : d.ks;
        }
        int ct_h = 0, ct_j = 0, ct_k = 0;
        double ct_wj = 0.0, ct_wk = 0.0, ct_kb = 0.0, ct_phi = 0.0;
        if ((int)threadIdx.x < nt) {
            const int4 r = __ldg(m.tref + t0 + threadIdx.x);
            const int w = __ldg(&d.tri[r.w].w);
            ct_h = r.x;
            ct_j = r.y;
            ct_k = r.z;
            ct_wj = wrap_shift((signed char)(w & 0xff), W);
            ct_wk = wrap_shift((signed char)((w >> 8) & 0xff), W);
            ct_kb = d.tri_kb ? __ldg(d.tri_kb + r.w) : d.kb;
            ct_phi = d.tri_phi0 ? __ldg(d.tri_phi0 + r.w) : 0.0;
        }
        auto xaddr = [&](int ref) -> unsigned {
            const int sb = (int)((unsigned)ref >> 16), r = sb >> lg;
            const int local = (sb & ((1 << lg) - 1)) * bsub + (ref & 0xffff);
            return s_ax[r] + 16u * (unsigned)local;
        };
        auto bond_item = [&](int ri, int rj, double wW, double l0, double k) -> double2 {
            const double2 p1 = cl_ld2d(xaddr(ri)), p2 = cl_ld2d(xaddr(rj));
            double fx, fy;
            bond_force(p1.x, p1.y, p2.x, p2.y, wW, l0, k, fx, fy);
            return make_double2(fx, fy);
        };
        auto tri_item = [&](int rh, int rj, int rk, double wj, double wk, double kb, double phi0) -> double4 {
            const double2 ph = cl_ld2d(xaddr(rh)), pj = cl_ld2d(xaddr(rj)), pk = cl_ld2d(xaddr(rk));
            const double ax = (pj.x + wj) - ph.x, ay = pj.y - ph.y;
            const double bx = (pk.x + wk) - ph.x, by = pk.y - ph.y;
            double fjx, fjy, fkx, fky;
            bend_force(ax, ay, bx, by, kb, phi0, fjx, fjy, fkx, fky);
            return make_double4(fjx, fjy, fkx, fky);
        };
        bool init = true;
        for (;;) {
            if (!init) {
                /* pass A, own nodes */
                const Scal &s = s_sc;
                for (int li = threadIdx.x; li < nloc; li += blockDim.x) {
                    double2 xi = s_x[li], vi = s_v[li];
                    const double2 fi = s_f[li];
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
                        s_x[li] = xi;
                    }
                    s_v[li] = vi;
                }
                if (s.done) break;
            }
            cl.sync();
            /* item pass: own bonds and triples, positions of any CTA */
            if ((int)threadIdx.x < nb) s_bf[threadIdx.x] = bond_item(cb_i, cb_j, cb_w, cb_l0, cb_k);
            for (int k = threadIdx.x + blockDim.x; k < nb; k += blockDim.x) {
                const int2 r = __ldg(m.bref + b0 + k);
                const int b = __ldg(m.bidx + b0 + k);
                s_bf[k] = bond_item(r.x, r.y, wrap_shift(__ldg(&d.bond[b].z), W), __ldg(d.bond_l0 + b),
                                    d.bond_k ? __ldg(d.bond_k + b) : d.ks);
            }
            if ((int)threadIdx.x < nt) s_tf[threadIdx.x] = tri_item(ct_h, ct_j, ct_k, ct_wj, ct_wk, ct_kb, ct_phi);
            for (int k = threadIdx.x + blockDim.x; k < nt; k += blockDim.x) {
                const int4 r = __ldg(m.tref + t0 + k);
                const int w = __ldg(&d.tri[r.w].w);
                s_tf[k] = tri_item(r.x, r.y, r.z, wrap_shift((signed char)(w & 0xff), W),
                                   wrap_shift((signed char)((w >> 8) & 0xff), W), d.tri_kb ? __ldg(d.tri_kb + r.w) : d.kb,
                                   d.tri_phi0 ? __ldg(d.tri_phi0 + r.w) : 0.0);
            }
            cl.sync();
            /* gather, half kick (v = 0 at the start), chunk partials; warp w
             * takes the CTA's 32-node chunks w, w + 8, ... */
            const double dtm = init ? 0.0 : s_sc.dtm;
            const int nch = (nloc + kChunk - 1) / kChunk;
            for (int c = warp; c < nch; c += blockDim.x / 32) {
                const int li = c * kChunk + lane, i = n0 + li;
                double tP = 0.0, tV = 0.0, tF = 0.0;
                if (li < nloc) {
                    double fx = 0.0, fy = 0.0;
                    const unsigned fc = __ldg(d.fcode + i);
                    if (fc != 0) {
                        if (d.use_bonds) {
                            const int e1 = __ldg(d.bptr + i + 1);
                            for (int e = __ldg(d.bptr + i); e < e1; ++e) {
                                const unsigned code = (unsigned)__ldg(m.bent + e);
                                const int r = (int)(code >> 28) >> lg;
                                const int ls = (int)((code >> 1) & 0x7ffffffu) - m.bo[r * spr];
                                const double2 f = cl_ld2d(s_abf[r] + 16u * (unsigned)ls);
                                /* a select, not a branch: the same sum */
                                fx = fx + ((code & 1) ? -f.x : f.x);
                                fy = fy + ((code & 1) ? -f.y : f.y);
                            }
                        }
                        if (d.use_triples) {
                            const int e1 = __ldg(d.tptr + i + 1);
                            for (int e = __ldg(d.tptr + i); e < e1; ++e) {
                                const unsigned code = (unsigned)__ldg(m.tent + e);
                                const int r = (int)(code >> 28) >> lg;
                                const int role = code & 3;
                                const int ls = (int)((code >> 2) & 0x3ffffffu) - m.to[r * spr];
                                const double4 f = cl_ld4d(s_atf[r] + 32u * (unsigned)ls);
                                /* selects, not a branch per role: the same
                                 * operands and operations as the oracle's
                                 * case-by-case sum */
                                const double hx = (-f.x) - f.z, hy = (-f.y) - f.w;
                                fx = fx + (role == 0 ? hx : (role == 1 ? f.x : f.z));
                                fy = fy + (role == 0 ? hy : (role == 1 ? f.y : f.w));
                            }
                        }
                        if (!(fc & 1)) fx = 0.0;
                        if (!(fc & 2)) fy = 0.0;
                    }
                    double2 vi;
                    if (init) {
                        vi = make_double2(0.0, 0.0);
                    } else {
                        vi = s_v[li];
                        vi.x = fma(dtm, fx, vi.x);
                        vi.y = fma(dtm, fy, vi.y);
                    }
                    s_v[li] = vi;
                    s_f[li] = make_double2(fx, fy);
                    tP = dot2(vi.x, vi.y, fx, fy);
                    tV = dot2(vi.x, vi.y, vi.x, vi.y);
                    tF = dot2(fx, fy, fx, fy);
                }
                const double sP = warp_sum(tP), sV = warp_sum(tV), sF = warp_sum(tF), sM = warp_max(tF);
                if (lane == 0) {
                    s_part[c] = sP;
                    s_part[umax + c] = sV;
                    s_part[2 * umax + c] = sF;
                    s_part[3 * umax + c] = sM;
                }
            }
            cl.sync();
            /* every CTA: the canonical totals over all chunks (units of one
             * chunk, padded with zeros to whole 256-node tiles), then the
             * FIRE scalars in thread 0 */
            auto unit = [&](int q, int u) -> double {
                if (u * kChunk >= d.n) return 0.0;
                const int r = (u * kChunk) / per, lc = u - r * (per / kChunk);
                return cl_ld1d(s_apt[r] + 8u * (unsigned)(q * umax + lc));
            };
            double tot[3];
            for (int q = 0; q < 3; ++q) {
                double acc = 0.0;
                const int k = 32 * warp + lane; /* 8 warps: lane sums of tiles k, k + 256, ... */
                for (int t = k; t < d.n_tiles; t += kTile) {
                    double u8[8];
                    for (int j = 0; j < 8; ++j) u8[j] = unit(q, 8 * t + j);
                    const double ts = ((u8[0] + u8[1]) + (u8[2] + u8[3])) + ((u8[4] + u8[5]) + (u8[6] + u8[7]));
                    acc = t == k ? ts : acc + ts;
                }
                acc = warp_sum(acc);
                if (lane == 0) s_red[8 * q + warp] = acc;
            }
            double mx = 0.0;
            for (int u = threadIdx.x; u < n_units; u += blockDim.x) mx = fmax(mx, unit(3, u));
            mx = warp_max(mx);
            if (lane == 0) s_red[24 + warp] = mx;
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int q = 0; q < 3; ++q) tot[q] = tree8(s_red + 8 * q);
                double M2 = s_red[24];
                for (int w = 1; w < 8; ++w) M2 = fmax(M2, s_red[24 + w]);
                if (init) scal_init(s_sc, p, tot[2], M2, d.sqrt_dof);
                else scal_step(s_sc, p, tot[0], tot[1], tot[2], M2, d.sqrt_dof);
            }
            __syncthreads();
            init = false;
        }
        /* the relaxed state out, energies over the cluster, report */
        for (int li = threadIdx.x; li < nloc; li += blockDim.x) {
            d.x[n0 + li] = s_x[li];
            d.v[n0 + li] = s_v[li];
            d.f[n0 + li] = s_f[li];
        }
        cl.sync();
        energy_tiles<false>(d, rank, C, s_red);
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

size_t dsm64_smem_bytes(int bmax, int emax, int tmax) { return dsm64_layout(Dsm64Sizes{bmax, emax, tmax}).total; }

static cudaError_t dsm64_config(int cluster, size_t smem, cudaLaunchConfig_t &cfg, cudaLaunchAttribute *attr,
                                int *max_clusters) {
    cudaError_t e;
    int dev, sms;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(k_fire_dsm64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) != cudaSuccess)
        return e;
    if (cluster > 8 &&
        (e = cudaFuncSetAttribute(k_fire_dsm64, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) != cudaSuccess)
        return e;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg = cudaLaunchConfig_t{};
    cfg.blockDim = dim3(kDsm64Threads);
    cfg.dynamicSmemBytes = smem;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3((sms / cluster) * cluster);
    *max_clusters = 0;
    return cudaOccupancyMaxActiveClusters(max_clusters, (void *)k_fire_dsm64, &cfg);
}

cudaError_t dsm64_max_active(int cluster, int bmax, int emax, int tmax, int *out) {
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    return dsm64_config(cluster, dsm64_smem_bytes(bmax, emax, tmax), cfg, attr, out);
}

cudaError_t launch_fp64_dsm(const NetDev *nets_dev, const NetDsm *dsm_dev, int n_nets, int cluster, int bmax,
                            int emax, int tmax, const FireParamsDev &p, int *queue_dev, const int *order_dev,
                            cudaStream_t stream) {
    if (cluster < 1 || cluster > kDsmParts || (kDsmParts % cluster) != 0) return cudaErrorInvalidValue;
    const Dsm64Sizes z{std::max(bmax, 1), std::max(emax, 1), std::max(tmax, 1)};
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[1];
    int max_clusters = 0;
    cudaError_t e = dsm64_config(cluster, dsm64_layout(z).total, cfg, attr, &max_clusters);
    if (e != cudaSuccess) return e;
    if (max_clusters < 1) return cudaErrorLaunchOutOfResources;
    cfg.gridDim = dim3(std::max(1, std::min(n_nets, max_clusters)) * cluster);
    cfg.stream = stream;
    if ((e = cudaMemsetAsync(queue_dev, 0, sizeof(int), stream)) != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, k_fire_dsm64, nets_dev, dsm_dev, n_nets, p, queue_dev, order_dev, z);
}

}  // namespace nr
