/*
 * Mixed-precision FIRE: FP32 bulk, FP64 anchors and certification.
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
#include <cooperative_groups.h>

#include "fire_common.cuh"
#include "fire_launch.h"

namespace nr {

constexpr float kAnchorF = 1.0e-4f;
constexpr int kMixThreads = 512;

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
    const float rl = sqrtf(fmaf(rx, rx, ry * ry));
    const float ral = sqrtf(fmaf(rax, rax, ray * ray));
    const float inv_rl = 1.0f / rl;
    const float dl = dd / (rl + ral);
    const float c1 = (dl + sk.x) * inv_rl;
    const float l0 = ral - sk.x;
    const float c2 = l0 * dl * inv_rl / ral;
    const float k = sk.y;
    return make_float2(k * fmaf(dx, c1, rax * c2), k * fmaf(dy, c1, ray * c2));
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
    const float dth = atan2f(im, re);
    const float ax = aax + dj.x, ay = aay + dj.y, bx = bax + dk.x, by = bay + dk.y;
    const float ia2 = 1.0f / fmaf(ax, ax, ay * ay), ib2 = 1.0f / fmaf(bx, bx, by * by);
    const float qa = fmaf(2.0f, da_dot, fmaf(dj.x, dj.x, dj.y * dj.y)) * ia2 / aa2;
    const float qb = fmaf(2.0f, db_dot, fmaf(dk.x, dk.x, dk.y * dk.y)) * ib2 / bb2;
    const float dgax = fmaf(-dj.y, ia2, aay * qa), dgay = fmaf(dj.x, ia2, -(aax * qa));
    const float dgbx = fmaf(-dk.y, ib2, bay * qb), dgby = fmaf(dk.x, ib2, -(bax * qb));
    const float gax = -ay * ia2, gay = ax * ia2, gbx = -by * ib2, gby = bx * ib2;
    dFj = make_float2(kap * fmaf(phia, dgax, dth * gax), kap * fmaf(phia, dgay, dth * gay));
    dFk = make_float2(-kap * fmaf(phia, dgbx, dth * gbx), -kap * fmaf(phia, dgby, dth * gby));
}

/* Displacement store: double-float xy per node, in shared or global memory. */
struct UView {
    float2 *hi, *lo;
    __device__ __forceinline__ float2 diff(int a, int b) const { /* u_a - u_b */
        const float2 ah = hi[a], al = lo[a], bh = hi[b], bl = lo[b];
        return make_float2(df_diff(ah.x, al.x, bh.x, bl.x), df_diff(ah.y, al.y, bh.y, bl.y));
    }
    /* u_a - u_b as a double-float (dh + dl), the hi difference taken exactly
     * with a two-sum. */
    __device__ __forceinline__ void diff2(int a, int b, float2 &dh, float2 &dl) const {
        const float2 ah = hi[a], al = lo[a], bh = hi[b], bl = lo[b];
        float sx = ah.x - bh.x, bbx = sx - ah.x;
        float ex = (ah.x - (sx - bbx)) + (-bh.x - bbx);
        float sy = ah.y - bh.y, bby = sy - ah.y;
        float ey = (ah.y - (sy - bby)) + (-bh.y - bby);
        dh = make_float2(sx, sy);
        dl = make_float2(ex + (al.x - bl.x), ey + (al.y - bl.y));
    }
};

/* FP32 force change since the anchor for node i, gathered from the item
 * results bdf/tdf in incidence order; mag = sum of the entries' |df|. */
__device__ __forceinline__ float2 node_dforce(const NetDev &d, int i, float &mag) {
    float2 F = make_float2(0.f, 0.f);
    mag = 0.f;
    if (d.use_bonds) {
        const int e1 = d.bptr[i + 1];
#pragma unroll 4
        for (int e = d.bptr[i]; e < e1; ++e) {
            const int code = d.bent[e];
            float2 df = d.bdf[code >> 1];
            if (code & 1) df = make_float2(-df.x, -df.y);
            F.x += df.x;
            F.y += df.y;
            mag += fabsf(df.x) + fabsf(df.y);
        }
    }
    if (d.use_triples) {
        const int e1 = d.tptr[i + 1];
#pragma unroll 4
        for (int e = d.tptr[i]; e < e1; ++e) {
            const int code = d.tent[e];
            const int role = code & 3;
            const float4 q = d.tdf[code >> 2];
            float gx, gy, m;
            if (role == 0) {
                gx = -(q.x + q.z);
                gy = -(q.y + q.w);
                m = fabsf(q.x) + fabsf(q.y) + fabsf(q.z) + fabsf(q.w);
            } else {
                gx = role == 1 ? q.x : q.z;
                gy = role == 1 ? q.y : q.w;
                m = fabsf(gx) + fabsf(gy);
            }
            F.x += gx;
            F.y += gy;
            mag += m;
        }
    }
    return F;
}

/* Item pass (FP32): the force change of every bond on its node i and of
 * every triple on its nodes j and k, each computed once, by the team's
 * threads in item order. */
__device__ void mixed_items(const NetDev &d, int first, int stride, const UView &u) {
    if (d.use_bonds)
        for (int b = first; b < d.n_edges; b += stride) {
            const int4 r = d.bond[b];
            float2 dh, dlo;
            u.diff2(r.y, r.x, dh, dlo);
            d.bdf[b] = bond_dforce(d.mb_data[b], d.mb_sk[b], dh, dlo);
        }
    if (d.use_triples)
        for (int t = first; t < d.n_triples; t += stride) {
            const int4 r = d.tri[t];
            float2 dFj, dFk;
            tri_dforce(d.mt_arms[t], d.mt_pk[t], u.diff(r.y, r.x), u.diff(r.z, r.x), dFj, dFk);
            d.tdf[t] = make_float4(dFj.x, dFj.y, dFk.x, dFk.y);
        }
}

struct Team {
    int rank, size;
    __device__ int first() const { return rank * blockDim.x + threadIdx.x; }
    __device__ int stride() const { return size * blockDim.x; }
};

/* FP32 coefficients of the FIRE scalars the passes need; one thread owns
 * the FP64 scalars (Scal) and broadcasts these through shared memory, so
 * the CTA's other threads issue no FP64 work outside anchors. */
struct Coef {
    float na, a, dt, dtsq, dtm;
    int mix_pending, zero_v, done, anchor;
};
__device__ __forceinline__ void coef_from(Coef &c, const Scal &s, int anchor) {
    c.na = (float)s.mix_na;
    c.a = (float)s.mix_a;
    c.dt = (float)s.dt;
    c.dtsq = (float)s.dtsq;
    c.dtm = (float)s.dtm;
    c.mix_pending = s.mix_pending;
    c.zero_v = s.zero_v;
    c.done = s.done;
    c.anchor = anchor;
}

/* Per-thread FP32 partials of pass B: sums of P = v.F, |v|^2, |F|^2 and
 * maxima of |F|^2 and of sum_b |df_b| (the FP32 error bound). */
struct Part {
    float P, V2, F2, M2, A;
};

/* Warp reduction of a Part in FP32; lane 0 stores it in slots[q * 32 + warp]. */
__device__ __forceinline__ void warp_part(Part t, float *slots) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        t.P += __shfl_xor_sync(kFull, t.P, off);
        t.V2 += __shfl_xor_sync(kFull, t.V2, off);
        t.F2 += __shfl_xor_sync(kFull, t.F2, off);
        t.M2 = fmaxf(t.M2, __shfl_xor_sync(kFull, t.M2, off));
        t.A = fmaxf(t.A, __shfl_xor_sync(kFull, t.A, off));
    }
    if (lane == 0) {
        slots[0 * 32 + warp] = t.P;
        slots[1 * 32 + warp] = t.V2;
        slots[2 * 32 + warp] = t.F2;
        slots[3 * 32 + warp] = t.M2;
        slots[4 * 32 + warp] = t.A;
    }
}

/* CTA totals of the warp slots, in FP64, by the calling thread. */
__device__ __forceinline__ void slots_total(const float *slots, double (&t)[5]) {
    const int nw = blockDim.x >> 5;
    for (int q = 0; q < 5; ++q) {
        double acc = slots[q * 32];
        for (int w = 1; w < nw; ++w) {
            const double v = slots[q * 32 + w];
            acc = q < 3 ? acc + v : fmax(acc, v);
        }
        t[q] = acc;
    }
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
__device__ void anchor_move(const NetDev &d, const Team &tm, const UView &u) {
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        const float2 h = u.hi[i], l = u.lo[i];
        double2 x = d.x[i];
        x.x = x.x + ((double)h.x + (double)l.x);
        x.y = x.y + ((double)h.y + (double)l.y);
        d.x[i] = x;
        u.hi[i] = make_float2(0.f, 0.f);
        u.lo[i] = make_float2(0.f, 0.f);
    }
}

/* Anchor step 2 (after a team sync): the FP32 anchor record of every bond
 * and triple from FP64 geometry, the FP64 forces into f and the
 * double-float anchor force, ff = F; CTA partials of |F|^2 and max|F|^2. */
__device__ void anchor_eval(const NetDev &d, const Team &tm, double &F2, double &M2) {
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
        node_force_fp64(d, i, fx, fy);
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
__device__ void mixed_pass_a(const NetDev &d, const Team &tm, const Coef &c, const UView &u) {
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
            float2 h = u.hi[i], l = u.lo[i];
            df_add(h.x, l.x, fmaf(c.dt, v.x, c.dtsq * F.x));
            df_add(h.y, l.y, fmaf(c.dt, v.y, c.dtsq * F.y));
            u.hi[i] = h;
            u.lo[i] = l;
            v.x = fmaf(c.dtm, F.x, v.x);
            v.y = fmaf(c.dtm, F.y, v.y);
        }
        d.vf[i] = v;
    }
}

/* Pass B, gather (FP32, after the item pass and a team sync): F = F(X) + dF,
 * half kick, partials {P, V2, F2 | maxF2, max_i sum |df|} (the last bounds
 * the FP32 error of the difference sum). */
__device__ Part mixed_pass_b(const NetDev &d, const Team &tm, float dtm) {
    float P = 0.f, V2 = 0.f, F2 = 0.f, M2 = 0.f, A = 0.f;
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        const unsigned c = d.fcode[i];
        float2 F = make_float2(0.f, 0.f);
        if (c != 0) {
            float mag;
            const float2 dF = node_dforce(d, i, mag);
            A = fmaxf(A, mag);
            const float2 ah = d.fa_hi[i], al = d.fa_lo[i];
            F.x = ah.x + (al.x + dF.x);
            F.y = ah.y + (al.y + dF.y);
            if (!(c & 1)) F.x = 0.f;
            if (!(c & 2)) F.y = 0.f;
        }
        float2 v = d.vf[i];
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

__device__ void mixed_finish(const NetDev &d, const Team &tm) {
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        const float2 v = d.vf[i];
        d.v[i] = make_double2((double)v.x, (double)v.y);
    }
}

/* The anchor must move when the FP32 rounding of the difference sum,
 * about kErr * max_i sum_b |df_b|, is no longer small against the force the
 * run still has to resolve (the larger of max|F| and half the stop
 * threshold), or when max|F| has dropped far below the anchor force. */
constexpr double kErr = 2.0e-7;
__device__ __forceinline__ bool need_anchor(const Scal &s, const FireParamsDev &p, double M2, double Amax,
                                            double M2_anchor) {
    const double f = fmax(sqrt(M2), 0.5 * p.fcut);
    return s.converged || s.done || kErr * Amax > 0.1 * f ||
           M2 < (double)kAnchorF * (double)kAnchorF * M2_anchor;
}

/* After an anchor: the FP64 force decides convergence. */
__device__ __forceinline__ void certify(Scal &s, const FireParamsDev &p, double F2, double M2, double sqrt_dof) {
    s.fmag = sqrt(F2);
    s.maxf = sqrt(M2);
    s.converged = crit_met(p, s.fmag, s.maxf, sqrt_dof);
    if (!isfinite(s.fmag)) s.status = NR_ERR_NONFINITE;
    s.done = s.converged || s.step >= p.max_steps || s.status != 0;
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

__device__ void relax_network_cta_mixed(const NetDev &d, const FireParamsDev &p, float2 *s_u, int smem_nodes,
                                        MixShared &sh) {
    const Team tm{0, 1};
    UView u;
    if (d.n <= smem_nodes) {
        u.hi = s_u;
        u.lo = s_u + smem_nodes;
    } else {
        u.hi = d.u_hi;
        u.lo = d.u_lo;
    }
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        u.hi[i] = make_float2(0.f, 0.f);
        u.lo[i] = make_float2(0.f, 0.f);
        d.vf[i] = make_float2(0.f, 0.f);
    }
    Scal s; /* meaningful in thread 0 only */
    int n_anchor = 1;
    double M2_anchor = 0.0, F2, M2, tF2, tM2;
    anchor_eval(d, tm, F2, M2);
    anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
    if (threadIdx.x == 0) {
        scal_init(s, p, tF2, tM2, d.sqrt_dof);
        M2_anchor = tM2;
        coef_from(sh.coef, s, 0);
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
        if (threadIdx.x == 0) {
            double t[5];
            slots_total(sh.slots, t);
            scal_step(s, p, t[0], t[1], t[2], t[3], d.sqrt_dof);
            coef_from(sh.coef, s, need_anchor(s, p, t[3], t[4], M2_anchor));
        }
        __syncthreads();
        if (sh.coef.anchor) {
            anchor_move(d, tm, u);
            __syncthreads();
            anchor_eval(d, tm, F2, M2);
            anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
            if (threadIdx.x == 0) {
                M2_anchor = tM2;
                n_anchor++;
                certify(s, p, tF2, tM2, d.sqrt_dof);
                coef_from(sh.coef, s, 0);
            }
            __syncthreads();
        }
    }
    mixed_finish(d, tm);
    __syncthreads();
    energy_tiles(d, 0, 1, sh.red);
    double es, eb;
    energy_final(d, sh.red, es, eb);
    if (threadIdx.x == 0) {
        scal_store(d.st, s);
        d.st->fp64_steps = n_anchor;
        d.st->e_stretch = es;
        d.st->e_bend = eb;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kMixThreads, 1) k_fire_batch_mixed(const NetDev *nets, int n_nets, FireParamsDev p,
                                                                     int *queue, const int *order, int smem_nodes) {
    extern __shared__ float2 s_u[];
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

/* A network relaxed by the C CTAs of one cluster (C SMs): nodes are split
 * over the CTAs (interleaved), u lives in global memory (L2-resident), the
 * hardware cluster barrier orders the passes, and each CTA's partial sums
 * are read by every other CTA through distributed shared memory.  Thread 0
 * of every CTA advances an identical copy of the FP64 FIRE scalars from the
 * same totals taken in the same rank order, so no broadcast is needed. */
__device__ void cluster_totals(cooperative_groups::cluster_group &cl, double *s_part, int nq, int nsum, double *t) {
    const int C = (int)cl.num_blocks();
    for (int q = 0; q < nq; ++q) t[q] = 0.0;
    for (int r = 0; r < C; ++r) {
        const double *rp = cl.map_shared_rank(s_part, r);
        for (int q = 0; q < nq; ++q) t[q] = q < nsum ? t[q] + rp[q] : fmax(t[q], rp[q]);
    }
}

__global__ void __launch_bounds__(kMixThreads, 1) k_fire_cluster_mixed(const NetDev *nets, int n_nets,
                                                                       FireParamsDev p, int *queue,
                                                                       const int *order) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    __shared__ MixShared sh;
    __shared__ NetDev s_d;
    __shared__ int s_slot;
    __shared__ double s_part[5];
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
        const UView u{d.u_hi, d.u_lo};
        for (int i = tm.first(); i < d.n; i += tm.stride()) {
            u.hi[i] = make_float2(0.f, 0.f);
            u.lo[i] = make_float2(0.f, 0.f);
            d.vf[i] = make_float2(0.f, 0.f);
        }
        Scal s; /* replicated in thread 0 of every CTA */
        int n_anchor = 1;
        double M2_anchor = 0.0, F2, M2, tF2, tM2;
        anchor_eval(d, tm, F2, M2);
        anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
        if (threadIdx.x == 0) {
            s_part[0] = tF2;
            s_part[1] = tM2;
        }
        cl.sync();
        if (threadIdx.x == 0) {
            double t[2];
            cluster_totals(cl, s_part, 2, 1, t);
            scal_init(s, p, t[0], t[1], d.sqrt_dof);
            M2_anchor = t[1];
            coef_from(sh.coef, s, 0);
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
            if (threadIdx.x == 0) {
                double t[5];
                slots_total(sh.slots, t);
                for (int q = 0; q < 5; ++q) s_part[q] = t[q];
            }
            cl.sync();
            if (threadIdx.x == 0) {
                double t[5];
                cluster_totals(cl, s_part, 5, 3, t);
                scal_step(s, p, t[0], t[1], t[2], t[3], d.sqrt_dof);
                coef_from(sh.coef, s, need_anchor(s, p, t[3], t[4], M2_anchor));
            }
            __syncthreads();
            if (sh.coef.anchor) {
                anchor_move(d, tm, u);
                cl.sync();
                anchor_eval(d, tm, F2, M2);
                anchor_reduce(F2, M2, sh.dslots, tF2, tM2);
                if (threadIdx.x == 0) {
                    s_part[0] = tF2;
                    s_part[1] = tM2;
                }
                cl.sync();
                if (threadIdx.x == 0) {
                    double t[2];
                    cluster_totals(cl, s_part, 2, 1, t);
                    M2_anchor = t[1];
                    n_anchor++;
                    certify(s, p, t[0], t[1], d.sqrt_dof);
                    coef_from(sh.coef, s, 0);
                }
                __syncthreads();
            }
        }
        mixed_finish(d, tm);
        cl.sync();
        if (rank == 0) {
            energy_tiles(d, 0, 1, sh.red);
            double es, eb;
            energy_final(d, sh.red, es, eb);
            if (threadIdx.x == 0) {
                scal_store(d.st, s);
                d.st->fp64_steps = n_anchor;
                d.st->e_stretch = es;
                d.st->e_bend = eb;
            }
        }
        cl.sync();
    }
}

/* CTAs per network for a batch: enough that the largest network has about
 * kNodesPerCta nodes per CTA, a power of two up to the portable cluster
 * size 8. */
constexpr int kNodesPerCta = 1536;
int mixed_cluster_size(int max_nodes) {
    int c = 1;
    while (c < 8 && c * kNodesPerCta < max_nodes) c *= 2;
    return c;
}

cudaError_t launch_mixed_cluster(const NetDev *nets_dev, int n_nets, int cluster, const FireParamsDev &p,
                                 int *queue_dev, const int *order_dev, cudaStream_t stream) {
    cudaError_t e;
    int dev, sms;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kMixThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3((sms / cluster) * cluster);
    int max_clusters = 0;
    if ((e = cudaOccupancyMaxActiveClusters(&max_clusters, (void *)k_fire_cluster_mixed, &cfg)) != cudaSuccess)
        return e;
    if (max_clusters < 1) return cudaErrorLaunchOutOfResources;
    const int clusters = std::max(1, std::min(n_nets, max_clusters));
    cfg.gridDim = dim3(clusters * cluster);
    if ((e = cudaMemsetAsync(queue_dev, 0, sizeof(int), stream)) != cudaSuccess) return e;
    return cudaLaunchKernelEx(&cfg, k_fire_cluster_mixed, nets_dev, n_nets, p, queue_dev, order_dev);
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

cudaError_t launch_mixed_batch(const NetDev *nets_dev, int n_nets, int max_nodes, const FireParamsDev &p,
                               int *queue_dev, const int *order_dev, cudaStream_t stream) {
    const int smem_nodes = mixed_smem_nodes(max_nodes);
    const size_t smem = (size_t)smem_nodes * 16;
    cudaError_t e = cudaFuncSetAttribute(k_fire_batch_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev, sms, per_sm = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fire_batch_mixed, kMixThreads, smem)) !=
        cudaSuccess)
        return e;
    const int blocks = std::max(1, std::min(n_nets, std::max(1, per_sm) * sms));
    if ((e = cudaMemsetAsync(queue_dev, 0, sizeof(int), stream)) != cudaSuccess) return e;
    k_fire_batch_mixed<<<blocks, kMixThreads, smem, stream>>>(nets_dev, n_nets, p, queue_dev, order_dev, smem_nodes);
    return cudaGetLastError();
}

/* ------------------------------------------------------------------ */
/* One network over the whole GPU (cooperative team of CTAs)            */
/* ------------------------------------------------------------------ */

/* Combines the CTA partials part[q * G + c] (q < nq) of all G CTAs in CTA
 * order: sums for q < nsum, maxima after.  Called by the last-arriving CTA. */
__device__ void team_totals(const double *part, int G, int nq, int nsum, double *out) {
    for (int q = 0; q < nq; ++q) {
        double acc = q < nsum ? 0.0 : 0.0;
        for (int c = 0; c < G; ++c) {
            const double v = __ldcg(part + (size_t)q * G + c);
            acc = q < nsum ? acc + v : fmax(acc, v);
        }
        out[q] = acc;
    }
}

__global__ void __launch_bounds__(kMixThreads, 1) k_fire_grid_mixed(NetDev d, FireParamsDev p,
                                                                    unsigned long long budget_ns) {
    __shared__ MixShared sh;
    const Team tm{(int)blockIdx.x, (int)gridDim.x};
    const unsigned G = gridDim.x;
    FireState *st = d.st;
    const UView u{d.u_hi, d.u_lo};
    bool last;
    Scal s; /* meaningful in thread 0 only */
    for (int i = tm.first(); i < d.n; i += tm.stride()) {
        u.hi[i] = make_float2(0.f, 0.f);
        u.lo[i] = make_float2(0.f, 0.f);
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
            team_totals(d.part, G, 2, 1, t);
            scal_init(s, p, t[0], t[1], d.sqrt_dof);
            scal_store(st, s);
            st->m2_anchor = t[1];
            st->fp64_steps = 1;
            st->anchor_now = 0;
        }
        barrier_release(st);
    }
    for (;;) {
        if (threadIdx.x == 0) {
            scal_load(s, st);
            coef_from(sh.coef, s, 0);
        }
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
        if (threadIdx.x == 0) {
            double t[5];
            slots_total(sh.slots, t);
            for (int q = 0; q < 5; ++q) d.part[(size_t)q * G + blockIdx.x] = t[q];
        }
        if (!barrier_arrive(st, G, budget_ns, last, 13)) return;
        if (last) {
            if (threadIdx.x == 0) {
                double t[5];
                team_totals(d.part, G, 5, 3, t);
                scal_step(s, p, t[0], t[1], t[2], t[3], d.sqrt_dof);
                const volatile FireState *vs = st;
                const double m2a = vs->m2_anchor;
                scal_store(st, s);
                st->anchor_now = need_anchor(s, p, t[3], t[4], m2a);
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
                    team_totals(d.part, G, 2, 1, t);
                    scal_load(s, st);
                    certify(s, p, t[0], t[1], d.sqrt_dof);
                    scal_store(st, s);
                    st->m2_anchor = t[1];
                    st->fp64_steps = st->fp64_steps + 1;
                    st->anchor_now = 0;
                }
                barrier_release(st);
            }
        }
    }
    mixed_finish(d, tm);
}

int mixed_grid_blocks(int n) {
    int dev, sms, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fire_grid_mixed, kMixThreads, 0) != cudaSuccess)
        return 0;
    const int want = (n + kMixThreads - 1) / kMixThreads;
    return std::max(1, std::min(want, per_sm * sms));
}

cudaError_t launch_mixed_grid(const NetDev &d, const FireParamsDev &p, int blocks, unsigned long long budget_ns,
                              cudaStream_t stream) {
    NetDev dd = d;
    FireParamsDev pp = p;
    unsigned long long bb = budget_ns;
    void *args[] = {&dd, &pp, &bb};
    return cudaLaunchCooperativeKernel((const void *)k_fire_grid_mixed, dim3(blocks), dim3(kMixThreads), args, 0,
                                       stream);
}

}  // namespace nr
