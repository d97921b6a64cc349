/*
 * FP64 device code shared by the plain FP64 kernels (fire_fp64.cu) and the
 * FP64 anchor evaluations of the mixed-precision kernels (fire_mixed.cu):
 * the canonical per-node force gather, the FIRE scalar update of
 * run_fire_md (large_strain_relax.cu:616-718) and the energy reductions.
 * Both translation units are compiled with --fmad=false, so this code has
 * the same bits in both.
 */
#ifndef NR_FIRE_COMMON_CUH
#define NR_FIRE_COMMON_CUH

#include "../../include/netrelax.h"
#include "canon_math.h"
#include "nr_device.cuh"

namespace nr {

constexpr int kGroup = 16; /* reduction units buffered in shared memory per flush */

__device__ __forceinline__ void node_force_fp64(const NetDev &d, int i, double &fx, double &fy) {
    fx = 0.0;
    fy = 0.0;
    const unsigned c = d.fcode[i];
    if (c == 0) return;
    const double W = d.width;
    if (d.use_bonds) {
        const int e1 = d.bptr[i + 1];
        for (int e = d.bptr[i]; e < e1; ++e) {
            const int code = d.bent[e];
            const int b = code >> 1;
            const int4 r = d.bond[b];
            const double2 p1 = d.x[r.x], p2 = d.x[r.y];
            const double k = d.bond_k ? d.bond_k[b] : d.ks;
            double bfx, bfy;
            bond_force(p1.x, p1.y, p2.x, p2.y, wrap_shift(r.z, W), d.bond_l0[b], k, bfx, bfy);
            if (code & 1) {
                fx = fx + (-bfx);
                fy = fy + (-bfy);
            } else {
                fx = fx + bfx;
                fy = fy + bfy;
            }
        }
    }
    if (d.use_triples) {
        const int e1 = d.tptr[i + 1];
        for (int e = d.tptr[i]; e < e1; ++e) {
            const int code = d.tent[e];
            const int t = code >> 2, role = code & 3;
            const int4 r = d.tri[t];
            const double2 ph = d.x[r.x], pj = d.x[r.y], pk = d.x[r.z];
            const int wj = (signed char)(r.w & 0xff), wk = (signed char)((r.w >> 8) & 0xff);
            const double ax = (pj.x + wrap_shift(wj, W)) - ph.x, ay = pj.y - ph.y;
            const double bx = (pk.x + wrap_shift(wk, W)) - ph.x, by = pk.y - ph.y;
            const double kb = d.tri_kb ? d.tri_kb[t] : d.kb;
            const double phi0 = d.tri_phi0 ? d.tri_phi0[t] : 0.0;
            double fjx, fjy, fkx, fky;
            bend_force(ax, ay, bx, by, kb, phi0, fjx, fjy, fkx, fky);
            if (role == 0) {
                fx = fx + ((-fjx) - fkx);
                fy = fy + ((-fjy) - fky);
            } else if (role == 1) {
                fx = fx + fjx;
                fy = fy + fjy;
            } else {
                fx = fx + fkx;
                fy = fy + fky;
            }
        }
    }
    if (!(c & 1)) fx = 0.0;
    if (!(c & 2)) fy = 0.0;
}

/* Item pass of the FP64 force: every bond force (the value its first
 * endpoint receives) and every triple's (F_j, F_k) computed ONCE into
 * scratch, items b = first, first + stride, ...  GB300's FP64 pipe is the
 * bound of the plain path, and the per-node gather below would otherwise
 * evaluate each bond twice and each triple three times. */
__device__ inline void items_pass(const NetDev &d, int first, int stride) {
    const double W = d.width;
    if (d.use_bonds)
        for (int b = first; b < d.n_edges; b += stride) {
            const int4 r = d.bond[b];
            const double2 p1 = d.x[r.x], p2 = d.x[r.y];
            const double k = d.bond_k ? d.bond_k[b] : d.ks;
            double fx, fy;
            bond_force(p1.x, p1.y, p2.x, p2.y, wrap_shift(r.z, W), d.bond_l0[b], k, fx, fy);
            d.bfrc[b] = make_double2(fx, fy);
        }
    if (d.use_triples)
        for (int t = first; t < d.n_triples; t += stride) {
            const int4 r = d.tri[t];
            const double2 ph = d.x[r.x], pj = d.x[r.y], pk = d.x[r.z];
            const int wj = (signed char)(r.w & 0xff), wk = (signed char)((r.w >> 8) & 0xff);
            const double ax = (pj.x + wrap_shift(wj, W)) - ph.x, ay = pj.y - ph.y;
            const double bx = (pk.x + wrap_shift(wk, W)) - ph.x, by = pk.y - ph.y;
            const double kb = d.tri_kb ? d.tri_kb[t] : d.kb;
            const double phi0 = d.tri_phi0 ? d.tri_phi0[t] : 0.0;
            double fjx, fjy, fkx, fky;
            bend_force(ax, ay, bx, by, kb, phi0, fjx, fjy, fkx, fky);
            d.tfrc[t] = make_double4(fjx, fjy, fkx, fky);
        }
}

/* Per-node gather of the item forces in the canonical order; the same bits
 * as node_force_fp64 (the same values summed in the same order). */
__device__ __forceinline__ void node_force_items(const NetDev &d, int i, double &fx, double &fy) {
    fx = 0.0;
    fy = 0.0;
    const unsigned c = d.fcode[i];
    if (c == 0) return;
    if (d.use_bonds) {
        const int e1 = d.bptr[i + 1];
        for (int e = d.bptr[i]; e < e1; ++e) {
            const int code = d.bent[e];
            const double2 f = d.bfrc[code >> 1];
            if (code & 1) {
                fx = fx + (-f.x);
                fy = fy + (-f.y);
            } else {
                fx = fx + f.x;
                fy = fy + f.y;
            }
        }
    }
    if (d.use_triples) {
        const int e1 = d.tptr[i + 1];
        for (int e = d.tptr[i]; e < e1; ++e) {
            const int code = d.tent[e];
            const double4 f = d.tfrc[code >> 2];
            const int role = code & 3;
            if (role == 0) {
                fx = fx + ((-f.x) - f.z);
                fy = fy + ((-f.y) - f.w);
            } else if (role == 1) {
                fx = fx + f.x;
                fy = fy + f.y;
            } else {
                fx = fx + f.z;
                fy = fy + f.w;
            }
        }
    }
    if (!(c & 1)) fx = 0.0;
    if (!(c & 2)) fy = 0.0;
}

/* FIRE scalars, advanced identically by whoever holds them. */
struct Scal {
    double dt, dtm, dtsq, alpha, mix_na, mix_a, fmag, maxf, power, vmag;
    int mix_pending, zero_v, since, step, done, converged, status;
};

__device__ __forceinline__ bool crit_met(const FireParamsDev &p, double fmag, double maxf, double sqrt_dof) {
    return p.criterion == 1 ? (maxf < p.fcut) : (fmag / sqrt_dof < p.fcut);
}

/* State at the top of run_fire_md (large_strain_relax.cu:616-643). */
__device__ inline void scal_init(Scal &s, const FireParamsDev &p, double F2, double M2, double sqrt_dof) {
    s.alpha = p.alpha0;
    s.dt = p.dt_max;
    s.dtsq = .5 * s.dt * s.dt / p.mass;
    s.dtm = .5 * s.dt / p.mass;
    s.mix_na = 0.0;
    s.mix_a = 0.0;
    s.power = 0.0;
    s.vmag = 0.0;
    s.fmag = sqrt(F2);
    s.maxf = sqrt(M2);
    s.mix_pending = 0;
    s.zero_v = 0;
    s.since = 0;
    s.step = 0;
    s.converged = crit_met(p, s.fmag, s.maxf, sqrt_dof);
    s.status = isfinite(s.fmag) ? 0 : NR_ERR_NONFINITE;
    s.done = p.max_steps <= 0 || s.status != 0;
}

/* End of one loop iteration (large_strain_relax.cu:683-718): mixing
 * coefficients with the current alpha, then the dt / alpha adaption, then
 * the convergence test. */
__device__ inline void scal_step(Scal &s, const FireParamsDev &p, double P, double V2, double F2, double M2,
                          double sqrt_dof) {
    s.step++;
    s.power = P;
    s.vmag = sqrt(V2);
    s.fmag = sqrt(F2);
    s.maxf = sqrt(M2);
    s.mix_a = s.alpha * s.vmag / s.fmag;
    s.mix_na = -s.alpha;
    s.mix_pending = 1;
    if (P > 0) {
        s.since++;
        if (s.since > p.nmin) {
            s.dt = fmin(s.dt * p.finc, p.dt_max);
            s.dtm = .5 * s.dt / p.mass;
            s.dtsq = .5 * s.dt * s.dt / p.mass;
            s.alpha *= p.falpha;
        }
        s.zero_v = 0;
    } else {
        s.since = 0;
        s.dt *= p.fdec;
        s.dtm = .5 * s.dt / p.mass;
        s.dtsq = s.dt * s.dt * .5 / p.mass;
        s.alpha = p.alpha0;
        s.zero_v = 1;
    }
    s.converged = crit_met(p, s.fmag, s.maxf, sqrt_dof);
    if (!isfinite(s.fmag) || !isfinite(s.power)) s.status = NR_ERR_NONFINITE;
    s.done = s.converged || s.step >= p.max_steps || s.status != 0;
}

__device__ __forceinline__ void scal_store(FireState *st, const Scal &s) {
    st->dt = s.dt; st->dtm = s.dtm; st->dtsq = s.dtsq; st->alpha = s.alpha;
    st->mix_na = s.mix_na; st->mix_a = s.mix_a;
    st->fmag = s.fmag; st->maxf = s.maxf; st->power = s.power; st->vmag = s.vmag;
    st->mix_pending = s.mix_pending; st->zero_v = s.zero_v; st->since = s.since; st->step = s.step;
    st->done = s.done; st->converged = s.converged; st->status = s.status;
}
__device__ __forceinline__ void scal_load(Scal &s, const FireState *st_) {
    const volatile FireState *st = st_;
    s.dt = st->dt; s.dtm = st->dtm; s.dtsq = st->dtsq; s.alpha = st->alpha;
    s.mix_na = st->mix_na; s.mix_a = st->mix_a;
    s.fmag = st->fmag; s.maxf = st->maxf; s.power = st->power; s.vmag = st->vmag;
    s.mix_pending = st->mix_pending; s.zero_v = st->zero_v; s.since = st->since; s.step = st->step;
    s.done = st->done; s.converged = st->converged; s.status = st->status;
}

/* Energy partials of bond tiles [t0, ...) and triple tiles, tiles of 256
 * items reduced by the CTA's first 256 threads (8 warps; s_red holds 8
 * doubles).  The CTA must have at least 256 threads; threads beyond the
 * first 256 only take part in the barriers. */
__device__ inline void energy_tiles(const NetDev &d, int t0, int tstride, double *s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool in_tile = threadIdx.x < kTile;
    const double W = d.width;
    const int tb = (d.n_edges + kTile - 1) / kTile, tt = (d.n_triples + kTile - 1) / kTile;
    const int total = (d.use_bonds ? tb : 0) + (d.use_triples ? tt : 0);
    for (int t = t0; t < total; t += tstride) {
        const bool is_bond = d.use_bonds && t < tb;
        const int tile = is_bond ? t : t - (d.use_bonds ? tb : 0);
        const int item = in_tile ? tile * kTile + threadIdx.x : (is_bond ? d.n_edges : d.n_triples);
        double e = 0.0;
        if (is_bond) {
            if (item < d.n_edges) {
                const int4 r = d.bond[item];
                const double2 p1 = d.x[r.x], p2 = d.x[r.y];
                const double k = d.bond_k ? d.bond_k[item] : d.ks;
                e = bond_energy(p1.x, p1.y, p2.x, p2.y, wrap_shift(r.z, W), d.bond_l0[item], k);
            }
        } else if (item < d.n_triples) {
            const int4 r = d.tri[item];
            const double2 ph = d.x[r.x], pj = d.x[r.y], pk = d.x[r.z];
            const int wj = (signed char)(r.w & 0xff), wk = (signed char)((r.w >> 8) & 0xff);
            const double ax = (pj.x + wrap_shift(wj, W)) - ph.x, ay = pj.y - ph.y;
            const double bx = (pk.x + wrap_shift(wk, W)) - ph.x, by = pk.y - ph.y;
            const double kb = d.tri_kb ? d.tri_kb[item] : d.kb;
            const double phi0 = d.tri_phi0 ? d.tri_phi0[item] : 0.0;
            e = bend_energy(ax, ay, bx, by, kb, phi0);
        }
        if (in_tile) { /* warp-uniform: kTile is a multiple of 32 */
            e = warp_sum(e);
            if (lane == 0) s_red[warp] = e;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            const size_t off = is_bond ? 0 : (size_t)(tb > tt ? tb : tt);
            d.epart[off + tile] = tree8(s_red);
        }
        __syncthreads();
    }
}

__device__ inline void energy_final(const NetDev &d, double *s_red, double &es, double &eb) {
    const int tb = (d.n_edges + kTile - 1) / kTile, tt = (d.n_triples + kTile - 1) / kTile;
    es = 0.0;
    eb = 0.0;
    if (d.use_bonds && d.n_edges > 0) es = final_sum(d.epart, tb, 8, s_red);
    if (d.use_triples && d.n_triples > 0) eb = final_sum(d.epart + (tb > tt ? tb : tt), tt, 8, s_red);
}

}  // namespace nr

#endif
