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

/* Deformation gradient of gel element e at the positions x
 * (network_mesh_relax.cu:716-719, the reference's association). */
__device__ __forceinline__ void gel_defgrad(const NetDev &d, int e, double &f11, double &f12, double &f21,
                                            double &f22) {
    const int4 el = d.gel->elem[e];
    const double *M = d.gel->elem_inv + 6 * (size_t)e;
    const double2 p1 = d.x[el.x], p2 = d.x[el.y], p3 = d.x[el.z];
    f11 = p1.x * M[0] + p2.x * M[2] + p3.x * M[4];
    f12 = p1.x * M[1] + p2.x * M[3] + p3.x * M[5];
    f21 = p1.y * M[0] + p2.y * M[2] + p3.y * M[4];
    f22 = p1.y * M[1] + p2.y * M[3] + p3.y * M[5];
}

/* gel_forces (network_mesh_relax.cu:702-751) of element e: for vertex r the
 * two terms the reference adds to the x force (dU/dF11, dU/dF12 parts) and
 * the two it adds to the y force, in its expression order. */
__device__ __forceinline__ double4 gel_terms(const NetDev &d, int e, int r, double du11, double du12, double du21,
                                             double du22) {
    const double *M = d.gel->elem_inv + 6 * (size_t)e;
    const double a = M[2 * r], b = M[2 * r + 1];
    return make_double4(du11 * a, du12 * b, du21 * a, du22 * b);
}
__device__ __forceinline__ void gel_du(const NetDev &d, int e, double &du11, double &du12, double &du21,
                                       double &du22) {
    double f11, f12, f21, f22;
    gel_defgrad(d, e, f11, f12, f21, f22);
    const NetGel &g = *d.gel;
    const double A = g.elem_area[e];
    const double smod = g.smod, bmod = g.bmod, dil = g.gdil;
    const double det = f11 * f22 - f12 * f21;
    const double coeff1 = -smod * A / det;
    double coeff2 = bmod * (dil + 1 - det) + smod * (f11 * f11 + f12 * f12 + f21 * f21 + f22 * f22) / (2 * det * det);
    coeff2 *= A;
    du11 = f11 * coeff1 + f22 * coeff2;
    du12 = f12 * coeff1 - f21 * coeff2;
    du21 = f21 * coeff1 - f12 * coeff2;
    du22 = f22 * coeff1 + f11 * coeff2;
}
/* gel_energy (network_mesh_relax.cu:674-699) of element e, as |e| for the
 * cublasDasum the reference sums it with. */
__device__ __forceinline__ double gel_energy_abs(const NetDev &d, int e) {
    double f11, f12, f21, f22;
    gel_defgrad(d, e, f11, f12, f21, f22);
    const NetGel &g = *d.gel;
    const double A = g.elem_area[e];
    const double smod = g.smod, bmod = g.bmod, dil = g.gdil;
    const double det = f11 * f22 - f12 * f21;
    double en = smod * A * ((f11 * f11 + f12 * f12 + f21 * f21 + f22 * f22) / det - 2) / 2;
    en += bmod * A * (det - 1 - dil) * (det - 1 - dil) / 2;
    return fabs(en);
}
/* Adds an element's terms to a node's force in the reference's atomicAdd
 * order (x: term 1 then term 2; y likewise). */
__device__ __forceinline__ void gel_add(double4 t, double &fx, double &fy) {
    fx = fx + t.x;
    fx = fx + t.y;
    fy = fy + t.z;
    fy = fy + t.w;
}

/* Masked force on node i from its bonds, triples and (kGel) gel elements,
 * in the canonical order.  The mixed-precision kernels never carry a gel
 * and instantiate kGel = false. */
template <bool kGel = true>
__device__ __forceinline__ void node_force_fp64_own(const NetDev &d, int i, double &fx, double &fy) {
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
    if (kGel && d.use_gel) {
        const NetGel &g = *d.gel;
        const int e1 = g.eptr[i + 1];
        for (int e = g.eptr[i]; e < e1; ++e) {
            const int code = g.eent[e];
            const int el = code / 3, r = code - 3 * el;
            double du11, du12, du21, du22;
            gel_du(d, el, du11, du12, du21, du22);
            gel_add(gel_terms(d, el, r, du11, du12, du21, du22), fx, fy);
        }
    }
    if (!(c & 1)) fx = 0.0;
    if (!(c & 2)) fy = 0.0;
}

/* Force on node i: its own masked sum plus, for a duplicate mesh vertex,
 * its partner's (duplicate_forces, network_mesh_relax.cu:754-780, unmasked;
 * a + b and b + a round alike, so both vertices get the same value). */
__device__ __forceinline__ void node_force_fp64(const NetDev &d, int i, double &fx, double &fy) {
    node_force_fp64_own(d, i, fx, fy);
    if (d.use_gel) {
        const int q = d.gel->partner[i];
        if (q >= 0) {
            double gx, gy;
            node_force_fp64_own(d, q, gx, gy);
            fx = fx + gx;
            fy = fy + gy;
        }
    }
}

/* Item pass of the FP64 force: every bond force (the value its first
 * endpoint receives) and every triple's (F_j, F_k) computed ONCE into
 * scratch, items b = first, first + stride, ...  GB300's FP64 pipe is the
 * bound of the plain path, and the per-node gather below would otherwise
 * evaluate each bond twice and each triple three times. */
template <bool kGel>
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
    if (kGel && d.use_gel)
        for (int e = first; e < d.n_elems; e += stride) {
            double du11, du12, du21, du22;
            gel_du(d, e, du11, du12, du21, du22);
            for (int r = 0; r < 3; ++r) d.gel->efrc[3 * (size_t)e + r] = gel_terms(d, e, r, du11, du12, du21, du22);
        }
}

/* Per-node gather of the item forces in the canonical order; the same bits
 * as node_force_fp64_own (the same values summed in the same order). */
template <bool kGel>
__device__ __forceinline__ void node_force_items_own(const NetDev &d, int i, double &fx, double &fy) {
    fx = 0.0;
    fy = 0.0;
    const unsigned c = d.fcode[i];
    if (c == 0) return;
    if (d.use_bonds) {
        const int e1 = d.bptr[i + 1];
        for (int e = d.bptr[i]; e < e1; ++e) {
            const int code = d.bent[e];
            const double2 f = d.bfrc[code >> 1];
            /* a select, not a branch: the same sum */
            fx = fx + ((code & 1) ? -f.x : f.x);
            fy = fy + ((code & 1) ? -f.y : f.y);
        }
    }
    if (d.use_triples) {
        const int e1 = d.tptr[i + 1];
        for (int e = d.tptr[i]; e < e1; ++e) {
            const int code = d.tent[e];
            const double4 f = d.tfrc[code >> 2];
            const int role = code & 3;
            /* selects, not a branch per role (lanes hold different roles):
             * the hinge takes -(F_j + F_k) as (-F_j) - F_k, j F_j, k F_k */
            const double hx = (-f.x) - f.z, hy = (-f.y) - f.w;
            fx = fx + (role == 0 ? hx : (role == 1 ? f.x : f.z));
            fy = fy + (role == 0 ? hy : (role == 1 ? f.y : f.w));
        }
    }
    if (kGel && d.use_gel) {
        const NetGel &g = *d.gel;
        const int e1 = g.eptr[i + 1];
        for (int e = g.eptr[i]; e < e1; ++e) gel_add(g.efrc[g.eent[e]], fx, fy);
    }
    if (!(c & 1)) fx = 0.0;
    if (!(c & 2)) fy = 0.0;
}

/* node_force_fp64 from the item scratch.  kGel = false compiles the gel
 * terms out (networks without a gel). */
template <bool kGel>
__device__ __forceinline__ void node_force_items(const NetDev &d, int i, double &fx, double &fy) {
    node_force_items_own<kGel>(d, i, fx, fy);
    if (kGel && d.use_gel) {
        const int q = d.gel->partner[i];
        if (q >= 0) {
            double gx, gy;
            node_force_items_own<kGel>(d, q, gx, gy);
            fx = fx + gx;
            fy = fy + gy;
        }
    }
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

/* Energy and virial partials of bond, triple and gel-element tiles (t0,
 * t0 + tstride, ... over the three lists in that order), tiles of 256 items
 * reduced by the CTA's first 256 threads (8 warps; s_red holds 32 doubles).
 * The CTA must have at least 256 threads; threads beyond the first 256 only
 * take part in the barriers.  Partial q of a tile goes to epart[q * M +
 * tile], M the largest tile count of the three lists: bonds E, W_xx, W_yy,
 * W_xy at q = 0..3, triples at 4..7, gel elements (energy only) at 8. */
__device__ __forceinline__ int energy_stride(const NetDev &d) {
    const int tb = (d.n_edges + kTile - 1) / kTile, tt = (d.n_triples + kTile - 1) / kTile;
    const int tg = (d.n_elems + kTile - 1) / kTile;
    return max(tb, max(tt, tg));
}

template <bool kGel = true>
__device__ inline void energy_tiles(const NetDev &d, int t0, int tstride, double *s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool in_tile = threadIdx.x < kTile;
    const double W = d.width;
    const int nb = d.use_bonds ? (d.n_edges + kTile - 1) / kTile : 0;
    const int nt = d.use_triples ? (d.n_triples + kTile - 1) / kTile : 0;
    const int ng = kGel && d.use_gel ? (d.n_elems + kTile - 1) / kTile : 0;
    const int total = nb + nt + ng;
    const size_t M = (size_t)energy_stride(d);
    for (int t = t0; t < total; t += tstride) {
        const int cat = t < nb ? 0 : (t < nb + nt ? 1 : 2);
        const int tile = cat == 0 ? t : (cat == 1 ? t - nb : t - nb - nt);
        const int n_items = cat == 0 ? d.n_edges : (cat == 1 ? d.n_triples : d.n_elems);
        const int item = in_tile ? tile * kTile + threadIdx.x : n_items;
        double e = 0.0, wxx = 0.0, wyy = 0.0, wxy = 0.0;
        if (item < n_items) {
            if (cat == 0) {
                const int4 r = d.bond[item];
                const double2 p1 = d.x[r.x], p2 = d.x[r.y];
                const double k = d.bond_k ? d.bond_k[item] : d.ks;
                const double wW = wrap_shift(r.z, W), l0 = d.bond_l0[item];
                e = bond_energy(p1.x, p1.y, p2.x, p2.y, wW, l0, k);
                bond_virial(p1.x, p1.y, p2.x, p2.y, wW, l0, k, wxx, wyy, wxy);
            } else if (cat == 1) {
                const int4 r = d.tri[item];
                const double2 ph = d.x[r.x], pj = d.x[r.y], pk = d.x[r.z];
                const int wj = (signed char)(r.w & 0xff), wk = (signed char)((r.w >> 8) & 0xff);
                const double ax = (pj.x + wrap_shift(wj, W)) - ph.x, ay = pj.y - ph.y;
                const double bx = (pk.x + wrap_shift(wk, W)) - ph.x, by = pk.y - ph.y;
                const double kb = d.tri_kb ? d.tri_kb[item] : d.kb;
                const double phi0 = d.tri_phi0 ? d.tri_phi0[item] : 0.0;
                e = bend_energy(ax, ay, bx, by, kb, phi0);
                bend_virial(ax, ay, bx, by, kb, phi0, wxx, wyy, wxy);
            } else if (kGel) {
                e = gel_energy_abs(d, item);
            }
        }
        if (in_tile) { /* warp-uniform: kTile is a multiple of 32 */
            e = warp_sum(e);
            wxx = warp_sum(wxx);
            wyy = warp_sum(wyy);
            wxy = warp_sum(wxy);
            if (lane == 0) {
                s_red[warp] = e;
                s_red[8 + warp] = wxx;
                s_red[16 + warp] = wyy;
                s_red[24 + warp] = wxy;
            }
        }
        __syncthreads();
        if (threadIdx.x < 4 && (cat < 2 || threadIdx.x == 0)) {
            const int q = cat == 2 ? 8 : 4 * cat + threadIdx.x;
            d.epart[(size_t)q * M + tile] = tree8(s_red + 8 * threadIdx.x);
        }
        __syncthreads();
    }
}

/* Totals of the energy pass: energies and the virial {W_xx, W_yy, W_xy}
 * (bond sum + triple sum; the gel contributes no virial). */
__device__ inline void energy_final(const NetDev &d, double *s_red, double &es, double &eb, double &eg,
                                    double *vir = nullptr) {
    const int tb = (d.n_edges + kTile - 1) / kTile, tt = (d.n_triples + kTile - 1) / kTile;
    const int tg = (d.n_elems + kTile - 1) / kTile;
    const size_t M = (size_t)energy_stride(d);
    es = 0.0;
    eb = 0.0;
    eg = 0.0;
    double wb[3] = {0.0, 0.0, 0.0}, wt[3] = {0.0, 0.0, 0.0};
    const bool bonds = d.use_bonds && d.n_edges > 0, tris = d.use_triples && d.n_triples > 0;
    if (bonds) es = final_sum(d.epart, tb, 8, s_red);
    if (tris) eb = final_sum(d.epart + 4 * M, tt, 8, s_red);
    if (d.use_gel && d.n_elems > 0) eg = final_sum(d.epart + 8 * M, tg, 8, s_red);
    if (vir) {
        for (int c = 0; c < 3; ++c) {
            if (bonds) wb[c] = final_sum(d.epart + (1 + c) * M, tb, 8, s_red);
            if (tris) wt[c] = final_sum(d.epart + (5 + c) * M, tt, 8, s_red);
            vir[c] = wb[c] + wt[c];
        }
    }
}

}  // namespace nr

#endif
