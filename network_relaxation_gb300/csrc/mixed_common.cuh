/*
 * Mixed-precision FIRE, shared device code: FP32 bulk, FP64 anchors and
 * certification.  The kernels are in fire_mixed.cu (CTA, cluster and grid
 * teams with state in global memory) and fire_dsm.cu (cluster teams with
 * the per-step state in distributed shared memory).
 *
 * GB300 runs FP32 about 64x faster than FP64, so the iteration runs in FP32
 * on displacements u = x - X from FP64 anchor positions X:
 *
 *   F(X + u) = F(X) + [F(X + u) - F(X)]
 *
 * F(X) is the canonical FP64 force (fire_common.cuh), kept per node as a
 * double-float (hi + lo FP32 pair).  The bracket is summed per node from
 * per-bond and per-triple FP32 DIFFERENCES whose rounding error is relative
 * to the difference itself:
 *   stretch  df = k [d (1 - l0/|r|) + l0 ra (|r| - |ra|) / (|r| |ra|)],
 *            r = ra + d, |r| - |ra| = (2 ra.d + d.d) / (|r| + |ra|)
 *   bending  dF_j = kb [phi_a dg(a) + dtheta g(a)], g(a) = perp(a)/|a|^2,
 *            dg(a) = perp(da)/|a|^2 - perp(a_a)(2 a_a.da + da.da)/(|a|^2|a_a|^2),
 *            dtheta = arg(conj(z_a) z_b), z_a = conj(a_a) a, z_b = conj(b_a) b
 * where ra, a_a, b_a, phi_a are the anchor's bond vectors and bend angle and
 * d, da, db the relative displacements.  u is a double-float too, so
 * d = u_j - u_i comes out with FP32 precision RELATIVE TO d (the hi parts of
 * neighbours subtract exactly), not relative to |u|.
 *
 * The anchor moves (X += u, u = 0, FP64 force and anchor data recomputed)
 * when the estimated FP32 rounding of the difference sum at some node,
 * kErr * sum_b |df_b|, exceeds a tenth of the force still to be resolved
 * (on soft modes bond-force changes can exceed the net force by 10^6), when
 * max|F| has dropped below kAnchorF * max|F(X)|, and whenever the FP32
 * force meets the stop criterion or the step cap is reached.  The run stops
 * as converged only when the FP64 force at the anchor meets the criterion,
 * so the returned positions are certified by the same FP64 force as the
 * plain path.
 *
 * Layout per network: u (hi, lo) lives in shared memory for the whole
 * relaxation when it fits (16 B/node), else in global memory; v, F and the
 * anchor force stream from global memory, coalesced (thread t owns nodes
 * t, t + blockDim, ...).  Pass B is item-centric: every bond and every
 * triple computes its force change ONCE, from its FP32 anchor record,
 *   bond    mb_data {ra hi.x, hi.y, lo.x, lo.y} (the anchor vector i -> j as
 *           a double-float), mb_sk {|ra| - l0, k}     -> bdf (change on i)
 *   triple  mt_arms {a_a, b_a}, mt_pk {phi_a, kb}     -> tdf (changes on j, k)
 * and after a team sync every node gathers its entries in incidence order
 * (bonds, then triples; a bond's second node takes -bdf, a hinge
 * -(dF_j + dF_k)).  Computing a bond from either end gives exactly opposite
 * FP32 results (round-to-nearest is odd-symmetric and every step of
 * bond_dforce is sign-covariant), so the gather reproduces a node-centric
 * evaluation bit for bit while doing a third of its arithmetic, free of the
 * warp divergence of per-entry roles.
 *
 * Compiled with --fmad=false (the FP64 anchor code stays canonical); FP32
 * expressions use explicit fmaf().
 */
#ifndef NR_MIXED_COMMON_CUH
#define NR_MIXED_COMMON_CUH

#include <cooperative_groups.h>

#include "fire_common.cuh"
#include "fire_launch.h"

namespace nr {

constexpr float kAnchorF = 1.0e-4f;
constexpr int kMixThreads = 512; /* grid kernel; batch and cluster kernels: 512 or 1024 */

/* Double-float helpers (Knuth two-sum). */
__device__ __forceinline__ void df_add(float &hi, float &lo, float x) {
    const float s = hi + x;
    const float bb = s - hi;
    const float err = (hi - (s - bb)) + (x - bb);
    const float l = lo + err;
    hi = s + l;
    lo = l - (hi - s);
}
/* (a_hi + a_lo) - (b_hi + b_lo) rounded to FP32. */
__device__ __forceinline__ float df_diff(float ah, float al, float bh, float bl) { return (ah - bh) + (al - bl); }

/* FP32 change of the stretch force on the entry's own node.  ra = anchor
 * vector self -> other as a double-float (hi, lo), sk = {|ra| - l0 (the
 * anchor strain, from FP64), k}, d = u_other - u_self as a double-float.
 *
 * On soft modes bonds mostly ROTATE: |d| is dominated by the component
 * perpendicular to the bond while the stretch |r| - |ra| that k multiplies
 * is tiny.  FP32 rounding of d or ra would leak ~6e-8 |d| of the
 * perpendicular part into the stretch, so |r|^2 - |ra|^2 = d.(2 ra + d) is
 * formed with exact products from the double-float pairs:
 *   |r| - |ra| = d.(2 ra + d) / (|r| + |ra|),  1 - l0/|r| = (|r| - |ra| + s_a) / |r|
 * and every remaining FP32 rounding is relative to the force change. */
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ float2 bond_dforce(float4 ra, float2 sk, float2 dh, float2 dlo) {
    const float rax = ra.x, ray = ra.y;
    /* |r|^2 - |ra|^2 = d.(2 ra + d).  Large rotations (floppy parts turn by
     * O(1) radians) make 2 ra.d and d.d cancel down to the stretch, so the
     * whole product is a double-float: w = 2 ra + d by two-sums, then exact
     * products of the hi parts and the cross terms. */
    float wxh, wxe, wyh, wye;
    two_sum(2.0f * rax, dh.x, wxh, wxe);
    two_sum(2.0f * ray, dh.y, wyh, wye);
    const float wxl = wxe + fmaf(2.0f, ra.z, dlo.x), wyl = wye + fmaf(2.0f, ra.w, dlo.y);
    const float p1 = dh.x * wxh, p2 = dh.y * wyh;
    const float e1 = fmaf(dh.x, wxh, -p1), e2 = fmaf(dh.y, wyh, -p2);
    float s, es;
    two_sum(p1, p2, s, es);
    const float lo = ((e1 + e2) + es) + (fmaf(dh.x, wxl, dh.y * wyl) + fmaf(dlo.x, wxh, dlo.y * wyh));
    const float dd = s + lo;
    const float dx = dh.x + dlo.x, dy = dh.y + dlo.y;
    const float rx = rax + dx, ry = ray + dy;
    /* hardware reciprocal square roots and an approximate quotient (a few
     * ulp): their error is relative to the force CHANGE, like every other
     * FP32 rounding here, and all of them are even in (ra, d) */
    const float q2 = fmaf(rx, rx, ry * ry), qa2 = fmaf(rax, rax, ray * ray);
    const float inv_rl = rsqrtf(q2), inv_ral = rsqrtf(qa2);
    const float rl = q2 * inv_rl, ral = qa2 * inv_ral;
    const float dl = __fdividef(dd, rl + ral);
    const float c1 = (dl + sk.x) * inv_rl;
    const float l0 = ral - sk.x;
    const float c2 = ((l0 * dl) * inv_rl) * inv_ral;
    const float k = sk.y;
    return make_float2(k * fmaf(dx, c1, rax * c2), k * fmaf(dy, c1, ray * c2));
}

/* atan2(im, re) for the bending-angle change since the anchor.  That
 * change is small in nearly every call (re > 0, |im| <= re / 8): there the
 * Taylor series atan t = t - t^3/3 + t^5/5 - t^7/7 + t^9/9 of t = im / re,
 * whose next term is below 1e-10 t, replaces the full-range function;
 * anything else goes to atan2f. */
__device__ __forceinline__ float small_atan2(float im, float re) {
    if (re > 0.0f && fabsf(im) <= 0.125f * re) {
        const float t = __fdividef(im, re), z = t * t;
        const float q = fmaf(fmaf(fmaf(fmaf(z, 1.0f / 9.0f, -1.0f / 7.0f), z, 1.0f / 5.0f), z, -1.0f / 3.0f), z, 0.0f);
        return fmaf(t, q, t);
    }
    return atan2f(im, re);
}

__device__ __forceinline__ void tri_dforce(float4 arms, float2 pk, float2 dj, float2 dk, float2 &dFj, float2 &dFk) {
    const float aax = arms.x, aay = arms.y, bax = arms.z, bay = arms.w;
    const float phia = pk.x, kap = pk.y;
    const float aa2 = fmaf(aax, aax, aay * aay), bb2 = fmaf(bax, bax, bay * bay);
    const float da_dot = fmaf(aax, dj.x, aay * dj.y), db_dot = fmaf(bax, dk.x, bay * dk.y);
    const float za_re = aa2 + da_dot, za_im = fmaf(aax, dj.y, -(aay * dj.x));
    const float zb_re = bb2 + db_dot, zb_im = fmaf(bax, dk.y, -(bay * dk.x));
    const float re = fmaf(zb_re, za_re, zb_im * za_im);
    const float im = fmaf(zb_im, za_re, -(zb_re * za_im));
    const float dth = small_atan2(im, re);
    const float ax = aax + dj.x, ay = aay + dj.y, bx = bax + dk.x, by = bay + dk.y;
    /* approximate reciprocals (a few ulp, relative to the change) */
    const float ia2 = __fdividef(1.0f, fmaf(ax, ax, ay * ay)), ib2 = __fdividef(1.0f, fmaf(bx, bx, by * by));
    const float qa = fmaf(2.0f, da_dot, fmaf(dj.x, dj.x, dj.y * dj.y)) * (ia2 * __fdividef(1.0f, aa2));
    const float qb = fmaf(2.0f, db_dot, fmaf(dk.x, dk.x, dk.y * dk.y)) * (ib2 * __fdividef(1.0f, bb2));
    const float dgax = fmaf(-dj.y, ia2, aay * qa), dgay = fmaf(dj.x, ia2, -(aax * qa));
    const float dgbx = fmaf(-dk.y, ib2, bay * qb), dgby = fmaf(dk.x, ib2, -(bax * qb));
    const float gax = -ay * ia2, gay = ax * ia2, gbx = -by * ib2, gby = bx * ib2;
    dFj = make_float2(kap * fmaf(phia, dgax, dth * gax), kap * fmaf(phia, dgay, dth * gay));
    dFk = make_float2(-kap * fmaf(phia, dgbx, dth * gbx), -kap * fmaf(phia, dgby, dth * gby));
}

/* u_a - u_b rounded to FP32 per component (u as double-float hi + lo). */
__device__ __forceinline__ float2 u_diff(float2 ah, float2 al, float2 bh, float2 bl) {
    return make_float2(df_diff(ah.x, al.x, bh.x, bl.x), df_diff(ah.y, al.y, bh.y, bl.y));
}
/* u_a - u_b as a double-float (dh + dl), the hi difference taken exactly
 * with a two-sum. */
__device__ __forceinline__ void u_diff2(float2 ah, float2 al, float2 bh, float2 bl, float2 &dh, float2 &dl) {
    float sx = ah.x - bh.x, bbx = sx - ah.x;
    float ex = (ah.x - (sx - bbx)) + (-bh.x - bbx);
    float sy = ah.y - bh.y, bby = sy - ah.y;
    float ey = (ah.y - (sy - bby)) + (-bh.y - bby);
    dh = make_float2(sx, sy);
    dl = make_float2(ex + (al.x - bl.x), ey + (al.y - bl.y));
}

/* Displacement store: double-float xy per node, {hi.x, hi.y, lo.x, lo.y},
 * in shared or global memory (one 16-byte access per node). */
struct UView {
    float4 *u;
    __device__ __forceinline__ float2 diff(int a, int b) const { /* u_a - u_b */
        const float4 ua = u[a], ub = u[b];
        return u_diff(make_float2(ua.x, ua.y), make_float2(ua.z, ua.w), make_float2(ub.x, ub.y),
                      make_float2(ub.z, ub.w));
    }
    __device__ __forceinline__ void diff2(int a, int b, float2 &dh, float2 &dl) const {
        const float4 ua = u[a], ub = u[b];
        u_diff2(make_float2(ua.x, ua.y), make_float2(ua.z, ua.w), make_float2(ub.x, ub.y), make_float2(ub.z, ub.w),
                dh, dl);
    }
};

/* -v when the entry's role bit is set, else v: the sign bit flipped
 * exactly, without a branch (the lanes of a warp hold different roles). */
__device__ __forceinline__ float2 neg_if(float2 v, unsigned code) {
    const unsigned sg = (code & 1u) << 31;
    return make_float2(__uint_as_float(__float_as_uint(v.x) ^ sg), __uint_as_float(__float_as_uint(v.y) ^ sg));
}

/* A triple entry's FP32 force change on its node, q = the triple's
 * {dF_j, dF_k}: role 0 (the hinge) -(dF_j + dF_k), role 1 dF_j, role 2
 * dF_k; m = the sum of the |components| involved.  Selects instead of a
 * branch per role (the lanes of a warp hold different roles), with the
 * case-by-case form's values and summation order. */
__device__ __forceinline__ void tri_entry(const float4 q, int role, float &gx, float &gy, float &m) {
    const bool h = role == 0, k2 = role == 2;
    const float sx = (k2 ? q.z : q.x) + (h ? q.z : 0.f);
    const float sy = (k2 ? q.w : q.y) + (h ? q.w : 0.f);
    gx = h ? -sx : sx;
    gy = h ? -sy : sy;
    const float ax = fabsf(q.x), ay = fabsf(q.y), az = fabsf(q.z), aw = fabsf(q.w);
    m = (((k2 ? az : ax) + (k2 ? aw : ay)) + (h ? az : 0.f)) + (h ? aw : 0.f);
}

/* FP32 force change since the anchor for node i, gathered from the item
 * results bdf/tdf in incidence order; mag = sum of the entries' |df|. */
__device__ __forceinline__ float2 node_dforce(const NetDev &d, int i, float &mag) {
    float2 F = make_float2(0.f, 0.f);
    mag = 0.f;
    if (d.use_bonds) {
        const int e1 = __ldg(d.bptr + i + 1);
#pragma unroll 4
        for (int e = __ldg(d.bptr + i); e < e1; ++e) {
            const int code = __ldg(d.bent + e);
            float2 df = d.bdf[code >> 1];
            df = neg_if(df, (unsigned)code);
            F.x += df.x;
            F.y += df.y;
            mag += fabsf(df.x) + fabsf(df.y);
        }
    }
    if (d.use_triples) {
        const int e1 = __ldg(d.tptr + i + 1);
#pragma unroll 4
        for (int e = __ldg(d.tptr + i); e < e1; ++e) {
            const int code = __ldg(d.tent + e);
            const int role = code & 3;
            const float4 q = d.tdf[code >> 2];
            float gx, gy, m;
            tri_entry(q, role, gx, gy, m);
            F.x += gx;
            F.y += gy;
            mag += m;
        }
    }
    return F;
}

/* Item pass (FP32): the force change of every bond on its node i and of
 * every triple on its nodes j and k, each computed once, by the team's
 * threads in item order.  Topology (bond, tri, the incidence lists, fcode)
 * never changes during a relaxation and is read through the read-only
 * cache; anchor records and u are rewritten in the kernel and are not. */
static __device__ void mixed_items(const NetDev &d, int first, int stride, const UView &u) {
    /* software pipelined: the next item's nodes and anchor record load
     * while the current item computes */
    if (d.use_bonds && first < d.n_edges) {
        int b = first;
        int4 r = __ldg(d.bond + b);
        float4 ra = d.mb_data[b];
        float2 sk = d.mb_sk[b];
        for (;;) {
            float2 dh, dlo;
            u.diff2(r.y, r.x, dh, dlo);
            const int nb = b + stride;
            int4 rn = r;
            float4 ran = ra;
            float2 skn = sk;
            if (nb < d.n_edges) {
                rn = __ldg(d.bond + nb);
                ran = d.mb_data[nb];
                skn = d.mb_sk[nb];
            }
            d.bdf[b] = bond_dforce(ra, sk, dh, dlo);
            if (nb >= d.n_edges) break;
            b = nb;
            r = rn;
            ra = ran;
            sk = skn;
        }
    }
    if (d.use_triples && first < d.n_triples) {
        int t = first;
        int4 r = __ldg(d.tri + t);
        float4 arms = d.mt_arms[t];
        float2 pk = d.mt_pk[t];
        for (;;) {
            const float2 dj = u.diff(r.y, r.x), dk = u.diff(r.z, r.x);
            const int nt = t + stride;
            int4 rn = r;
            float4 armsn = arms;
            float2 pkn = pk;
            if (nt < d.n_triples) {
                rn = __ldg(d.tri + nt);
                armsn = d.mt_arms[nt];
                pkn = d.mt_pk[nt];
            }
            float2 dFj, dFk;
            tri_dforce(arms, pk, dj, dk, dFj, dFk);
            d.tdf[t] = make_float4(dFj.x, dFj.y, dFk.x, dFk.y);
            if (nt >= d.n_triples) break;
            t = nt;
            r = rn;
            arms = armsn;
            pk = pkn;
        }
    }
}

struct Team {
    int rank, size;
    __device__ int first() const { return rank * blockDim.x + threadIdx.x; }
    __device__ int stride() const { return size * blockDim.x; }
};

/* Per-thread FP32 partials of pass B: sums of P = v.F, |v|^2, |F|^2 and
 * maxima of |F|^2 and of sum_b |df_b| (the FP32 error bound). */
struct Part {
    float P, V2, F2, M2, A;
};

/* Xor butterfly over the warp (fixed order: every lane ends with the same
 * totals, and equal inputs give equal totals in every CTA). */
__device__ __forceinline__ Part warp_reduce(Part t) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        t.P += __shfl_xor_sync(kFull, t.P, off);
        t.V2 += __shfl_xor_sync(kFull, t.V2, off);
        t.F2 += __shfl_xor_sync(kFull, t.F2, off);
        t.M2 = fmaxf(t.M2, __shfl_xor_sync(kFull, t.M2, off));
        t.A = fmaxf(t.A, __shfl_xor_sync(kFull, t.A, off));
    }
    return t;
}

/* Warp totals of a Part; lane 0 stores them in slots[q * 32 + warp]. */
__device__ __forceinline__ void warp_part(Part t, float *slots) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    t = warp_reduce(t);
    if (lane == 0) {
        slots[0 * 32 + warp] = t.P;
        slots[1 * 32 + warp] = t.V2;
        slots[2 * 32 + warp] = t.F2;
        slots[3 * 32 + warp] = t.M2;
        slots[4 * 32 + warp] = t.A;
    }
}

/* CTA totals of the warp slots, computed by warp 0 (lane w takes warp w's
 * slot); every lane of warp 0 returns them. */
__device__ __forceinline__ Part block_totals(const float *slots) {
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    Part t{0.f, 0.f, 0.f, 0.f, 0.f};
    if (lane < nw) t = Part{slots[lane], slots[32 + lane], slots[64 + lane], slots[96 + lane], slots[128 + lane]};
    return warp_reduce(t);
}

/* ----- FIRE scalars (large_strain_relax.cu:683-718) in FP32 -----
 *
 * The scalar update after each reduction is a serial chain that the whole
 * team waits for, and FP64 issues at 1/64 of the FP32 rate on this GPU: in
 * FP64 it took several microseconds per step.  The mixed path therefore
 * runs it in FP32 on the FP32 totals (the forces it acts on are FP32
 * already).  FP64 stays where the result is certified: |F| and max|F| from
 * the anchors, and the stop decision. */
struct MixParams {
    float alpha0, falpha, dt_max, finc, fdec, half_inv_m;
    float thr2;      /* stop threshold on the |F|^2 total (RMS) or on max |F|^2 */
    float half_fcut;
    int nmin, max_steps, crit_max;
};

__device__ __forceinline__ MixParams mix_params(const FireParamsDev &p, double sqrt_dof) {
    MixParams q;
    q.alpha0 = (float)p.alpha0;
    q.falpha = (float)p.falpha;
    q.dt_max = (float)p.dt_max;
    q.finc = (float)p.finc;
    q.fdec = (float)p.fdec;
    q.half_inv_m = (float)(0.5 / p.mass);
    const double thr = p.criterion == 1 ? p.fcut : p.fcut * sqrt_dof;
    q.thr2 = (float)(thr * thr);
    q.half_fcut = (float)(0.5 * p.fcut);
    q.nmin = p.nmin;
    q.max_steps = p.max_steps;
    q.crit_max = p.criterion == 1;
    return q;
}

/* State at the top of run_fire_md (large_strain_relax.cu:616-643); the
 * first anchor's certification follows. */
__device__ __forceinline__ void mix_init(MixScal &s, const MixParams &q) {
    s.dt = q.dt_max;
    s.dtm = s.dt * q.half_inv_m;
    s.dtsq = s.dt * s.dtm;
    s.alpha = q.alpha0;
    s.na = 0.f;
    s.a = 0.f;
    s.m2_anchor = 0.f;
    s.pad0 = 0.f;
    s.since = 0;
    s.step = 0;
    s.mix_pending = 0;
    s.zero_v = 0;
    s.done = 0;
    s.converged = 0;
    s.status = 0;
    s.n_anchor = 0;
    s.fmag = 0.0;
    s.maxf = 0.0;
}

/* End of one loop iteration: mixing coefficients with the current alpha,
 * dt / alpha adaption, the (FP32) stop test that claims convergence. */
__device__ __forceinline__ void mix_step(MixScal &s, const MixParams &q, const Part &t) {
    s.step++;
    s.a = s.alpha * sqrtf(t.V2) / sqrtf(t.F2);
    s.na = -s.alpha;
    s.mix_pending = 1;
    if (t.P > 0.f) {
        if (++s.since > q.nmin) {
            s.dt = fminf(s.dt * q.finc, q.dt_max);
            s.alpha *= q.falpha;
        }
        s.zero_v = 0;
    } else {
        s.since = 0;
        s.dt *= q.fdec;
        s.alpha = q.alpha0;
        s.zero_v = 1;
    }
    s.dtm = s.dt * q.half_inv_m;
    s.dtsq = s.dt * s.dtm;
    s.converged = (q.crit_max ? t.M2 : t.F2) < q.thr2;
    if (!isfinite(t.F2) || !isfinite(t.P)) s.status = NR_ERR_NONFINITE;
    s.done = s.converged || s.step >= q.max_steps || s.status != 0;
}

/* The anchor must move when the FP32 rounding of the difference sum,
 * about kErr * max_i sum_b |df_b|, is no longer small against the force the
 * run still has to resolve (the larger of max|F| and half the stop
 * threshold), when max|F| has dropped far below the anchor force, and
 * whenever the FP32 step claims convergence or ends the run. */
constexpr float kErr = 2.0e-7f;
__device__ __forceinline__ bool need_anchor(const MixScal &s, const MixParams &q, const Part &t) {
    const float f = fmaxf(sqrtf(t.M2), q.half_fcut);
    return s.converged || s.done || kErr * t.A > 0.1f * f || t.M2 < kAnchorF * kAnchorF * s.m2_anchor;
}

/* After an anchor: the FP64 totals at the anchor decide convergence (at
 * step 0 only the step cap and a non-finite force stop the run: the
 * reference always takes a first step). */
__device__ __forceinline__ void mix_certify(MixScal &s, const FireParamsDev &p, double sqrt_dof, double F2,
                                            double M2) {
    s.fmag = sqrt(F2);
    s.maxf = sqrt(M2);
    s.m2_anchor = (float)M2;
    s.n_anchor++;
    s.converged = crit_met(p, s.fmag, s.maxf, sqrt_dof);
    if (!isfinite(s.fmag)) s.status = NR_ERR_NONFINITE;
    s.done = (s.step > 0 && s.converged) || s.step >= p.max_steps || s.status != 0;
}

/* Report fields of the network's FireState. */
__device__ __forceinline__ void mix_report(FireState *st, const MixScal &s) {
    st->fmag = s.fmag;
    st->maxf = s.maxf;
    st->step = s.step;
    st->status = s.status;
    st->converged = s.converged;
    st->done = s.done;
    st->fp64_steps = s.n_anchor;
    st->dt = s.dt;
    st->alpha = s.alpha;
}

/* MixScal of a multi-CTA team, read from L2 after a grid barrier. */
__device__ __forceinline__ MixScal mix_load(const FireState *st) {
    static_assert(sizeof(MixScal) == 80, "MixScal is five 16-byte words");
    union {
        MixScal s;
        int4 w[5];
    } u;
    const int4 *src = reinterpret_cast<const int4 *>(&st->mix);
#pragma unroll
    for (int k = 0; k < 5; ++k) u.w[k] = __ldcg(src + k);
    return u.s;
}

/* FP32 coefficients of the next pass A, broadcast through shared memory. */
struct Coef {
    float na, a, dt, dtsq, dtm;
    int mix_pending, zero_v, done, anchor;
};
__device__ __forceinline__ Coef coef_of(const MixScal &s, int anchor) {
    return Coef{s.na, s.a, s.dt, s.dtsq, s.dtm, s.mix_pending, s.zero_v, s.done, anchor};
}

/* CTA totals of per-thread FP64 anchor partials (sum of F2, max of M2);
 * valid in thread 0 after the call.  dslots: 64 doubles. */
__device__ __forceinline__ void anchor_reduce(double F2, double M2, double *dslots, double &tF2, double &tM2) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int off = 16; off >= 1; off >>= 1) {
        F2 += __shfl_xor_sync(kFull, F2, off);
        M2 = fmax(M2, __shfl_xor_sync(kFull, M2, off));
    }
    if (lane == 0) {
        dslots[warp] = F2;
        dslots[32 + warp] = M2;
    }
    __syncthreads();
    tF2 = 0.0;
    tM2 = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < nw; ++w) {
            tF2 += dslots[w];
            tM2 = fmax(tM2, dslots[32 + w]);
        }
}

/* Anchor step 1: X += u (exactly, in FP64), u = 0. */
static __device__ void anchor_move(const NetDev &d, const Team &tm, const UView &u) {
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        const float4 w = u.u[i];
        const float2 h = make_float2(w.x, w.y), l = make_float2(w.z, w.w);
        double2 x = d.x[i];
        x.x = x.x + ((double)h.x + (double)l.x);
        x.y = x.y + ((double)h.y + (double)l.y);
        d.x[i] = x;
        u.u[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

/* Anchor step 2 (after a team sync): the FP32 anchor record of every bond
 * and triple from FP64 geometry, the FP64 forces into f and the
 * double-float anchor force, ff = F; CTA partials of |F|^2 and max|F|^2. */
static __device__ __noinline__ void anchor_eval(const NetDev &d, const Team &tm, double &F2, double &M2) {
    const double W = d.width;
    F2 = 0.0;
    M2 = 0.0;
    if (d.use_bonds)
        for (int b = tm.first(); b < d.n_edges; b += tm.stride()) {
            const int4 r = d.bond[b];
            const double2 p1 = d.x[r.x], p2 = d.x[r.y];
            const double rx = (p2.x + wrap_shift(r.z, W)) - p1.x, ry = p2.y - p1.y;
            const double k = d.bond_k ? d.bond_k[b] : d.ks;
            const float hx = (float)rx, hy = (float)ry;
            d.mb_data[b] = make_float4(hx, hy, (float)(rx - (double)hx), (float)(ry - (double)hy));
            d.mb_sk[b] = make_float2((float)(sqrt(fma(rx, rx, ry * ry)) - d.bond_l0[b]), (float)k);
        }
    if (d.use_triples)
        for (int t = tm.first(); t < d.n_triples; t += tm.stride()) {
            const int4 r = d.tri[t];
            const double2 ph = d.x[r.x], pj = d.x[r.y], pk = d.x[r.z];
            const int wj = (signed char)(r.w & 0xff), wk = (signed char)((r.w >> 8) & 0xff);
            const double ax = (pj.x + wrap_shift(wj, W)) - ph.x, ay = pj.y - ph.y;
            const double bx = (pk.x + wrap_shift(wk, W)) - ph.x, by = pk.y - ph.y;
            const double kb = d.tri_kb ? d.tri_kb[t] : d.kb;
            const double phi0 = d.tri_phi0 ? d.tri_phi0[t] : 0.0;
            d.mt_arms[t] = make_float4((float)ax, (float)ay, (float)bx, (float)by);
            d.mt_pk[t] = make_float2((float)bend_dtheta(ax, ay, bx, by, phi0), (float)kb);
        }
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        double fx, fy;
        node_force_fp64_own<false>(d, i, fx, fy);
        d.f[i] = make_double2(fx, fy);
        const float hx = (float)fx, hy = (float)fy;
        d.fa_hi[i] = make_float2(hx, hy);
        d.fa_lo[i] = make_float2((float)(fx - (double)hx), (float)(fy - (double)hy));
        d.ff[i] = make_float2(hx, hy);
        const double t = dot2(fx, fy, fx, fy);
        F2 += t;
        M2 = fmax(M2, t);
    }
}

/* Pass A (FP32): mixing / zeroing from the previous step, then drift. */
static __device__ void mixed_pass_a(const NetDev &d, const Team &tm, const Coef &c, const UView &u) {
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        float2 v = d.vf[i];
        const float2 F = d.ff[i];
        if (c.mix_pending) {
            v.x = fmaf(c.na, v.x, v.x);
            v.y = fmaf(c.na, v.y, v.y);
            v.x = fmaf(c.a, F.x, v.x);
            v.y = fmaf(c.a, F.y, v.y);
            if (c.zero_v) v = make_float2(0.f, 0.f);
        }
        if (!c.done) {
            float4 w = u.u[i];
            df_add(w.x, w.z, fmaf(c.dt, v.x, c.dtsq * F.x));
            df_add(w.y, w.w, fmaf(c.dt, v.y, c.dtsq * F.y));
            u.u[i] = w;
            v.x = fmaf(c.dtm, F.x, v.x);
            v.y = fmaf(c.dtm, F.y, v.y);
        }
        d.vf[i] = v;
    }
}

/* Pass B, gather (FP32, after the item pass and a team sync): F = F(X) + dF,
 * half kick, partials {P, V2, F2 | maxF2, max_i sum |df|} (the last bounds
 * the FP32 error of the difference sum). */
static __device__ Part mixed_pass_b(const NetDev &d, const Team &tm, float dtm) {
    float P = 0.f, V2 = 0.f, F2 = 0.f, M2 = 0.f, A = 0.f;
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        /* the node's independent loads first: one round trip */
        const unsigned c = __ldg(d.fcode + i);
        const float2 ah = d.fa_hi[i], al = d.fa_lo[i];
        float2 v = d.vf[i];
        float2 F = make_float2(0.f, 0.f);
        if (c != 0) {
            float mag;
            const float2 dF = node_dforce(d, i, mag);
            A = fmaxf(A, mag);
            F.x = ah.x + (al.x + dF.x);
            F.y = ah.y + (al.y + dF.y);
            if (!(c & 1)) F.x = 0.f;
            if (!(c & 2)) F.y = 0.f;
        }
        v.x = fmaf(dtm, F.x, v.x);
        v.y = fmaf(dtm, F.y, v.y);
        d.vf[i] = v;
        d.ff[i] = F;
        P += fmaf(v.x, F.x, v.y * F.y);
        V2 += fmaf(v.x, v.x, v.y * v.y);
        const float f2 = fmaf(F.x, F.x, F.y * F.y);
        F2 += f2;
        M2 = fmaxf(M2, f2);
    }
    return Part{P, V2, F2, M2, A};
}

static __device__ void mixed_finish(const NetDev &d, const Team &tm) {
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        const float2 v = d.vf[i];
        d.v[i] = make_double2((double)v.x, (double)v.y);
    }
}

/* ------------------------------------------------------------------ */
/* One CTA per network (batched)                                        */
/* ------------------------------------------------------------------ */

struct MixShared {
    float slots[5 * 32];
    double dslots[64];
    double red[32];
    Coef coef;
};

/* Canonical FP64 energies and virial of the network into st (one CTA).  Kept out of
 * line, like anchor_eval: the FP64 code's register demand stays out of the
 * FP32 loop. */
static __device__ __noinline__ void mixed_energies(const NetDev &d, double *s_red) {
    energy_tiles<false>(d, 0, 1, s_red);
    double es, eb, eg, vir[3];
    energy_final(d, s_red, es, eb, eg, vir);
    if (threadIdx.x == 0) {
        d.st->e_stretch = es;
        d.st->e_bend = eb;
        for (int c = 0; c < 3; ++c) d.st->vir[c] = vir[c];
    }
}

/* ----- distributed shared memory (thread-block clusters) ----- */

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
__device__ __forceinline__ void dsm_st1(unsigned a, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}
__device__ __forceinline__ void dsm_st1i(unsigned a, int v) {
    asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void dsm_st1d(unsigned a, double v) {
    asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
__device__ __forceinline__ float4 dsm_ld4(unsigned a) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(a));
    return v;
}

/* Cross-CTA totals are PUSHED: each CTA stores its value into its own slot
 * of every CTA's array before the cluster barrier that ends the phase (the
 * barrier's release / acquire orders the remote stores), and afterwards
 * every CTA reads the C slots from its own shared memory: no remote load
 * on the critical path after the barrier.  The next push into the same
 * slots comes after at least one more cluster barrier, which every CTA
 * reaches only after it has read them. */

/* Thread 0: this CTA's FP64 anchor totals into slot `rank` of s_ancs in
 * each of the cluster's C CTAs. */
__device__ __forceinline__ void anchor_push(double (*s_ancs)[2], int rank, int C, double tF2, double tM2) {
    for (int r = 0; r < C; ++r) {
        const unsigned a = dsm_addr(&s_ancs[rank][0], (unsigned)r);
        dsm_st1d(a, tF2);
        dsm_st1d(a + 8u, tM2);
    }
}

/* FP64 anchor totals (sum of F2, max of M2) over the ranks, in rank order,
 * from the pushed slots. */
__device__ __forceinline__ void anchor_totals(const double (*s_ancs)[2], int C, double *t) {
    t[0] = 0.0;
    t[1] = 0.0;
    for (int r = 0; r < C; ++r) {
        t[0] = t[0] + s_ancs[r][0];
        t[1] = fmax(t[1], s_ancs[r][1]);
    }
}

}  // namespace nr

#endif
