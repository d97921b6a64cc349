/*
 * Canonical FP64 arithmetic shared by the host builders and the CUDA kernels.
 *
 * Every rounding step is fixed: explicit fma() where a fused multiply-add is
 * wanted, separate operations everywhere else (host code is compiled with
 * -ffp-contract=off, device code with --fmad=false), and IEEE division and
 * square root only.  The same inputs therefore give the same bits on the GPU
 * and on any IEEE host, which is what lets the FP64 relaxation be compared
 * bit-for-bit with a CPU restatement.
 *
 * Formulas follow large_strain_relax.cu:
 *   stretch force   :386-414   F = ks (1 - l0/|r|) r, applied +F / -F
 *   bending force   :417-469   theta0 = pi, F_j = kb dth / |a|^2 (-a_y, a_x),
 *                              F_k = kb dth / |b|^2 (b_y, -b_x), hinge -(F_j+F_k)
 *   stretch energy  :472-490   ks/2 (|r| - l0)^2
 *   bending energy  :493-523   kb/2 (theta - pi)^2
 * with two deliberate differences: the bending angle uses nr_atan2 (below)
 * instead of libm/CUDA atan2, and theta - pi is formed as
 * atan2(-cross, -dot) rather than atan2(cross, dot) + 2pi - pi (the same
 * angle without the cancellation; it differs only for a fully folded triple).
 */
#ifndef NR_CANON_MATH_H
#define NR_CANON_MATH_H

#include <math.h>

#if defined(__CUDACC__)
#define NR_HD __host__ __device__ __forceinline__
#else
#define NR_HD inline
#endif

namespace nr {

/* atan(u) = u + u z Q(z), z = u^2 on |u| <= tan(pi/8); coefficients from
 * gen_atan_coeffs.py (Chebyshev interpolation in 60-digit arithmetic),
 * highest power first. */
#define NR_ATAN_Q0 (-0.01917688711906226)
#define NR_ATAN_Q1 (0.03923165829558719)
#define NR_ATAN_Q2 (-0.0508544973794026)
#define NR_ATAN_Q3 (0.0585814891280221)
#define NR_ATAN_Q4 (-0.06664511447381948)
#define NR_ATAN_Q5 (0.07692183190826087)
#define NR_ATAN_Q6 (-0.09090904578123903)
#define NR_ATAN_Q7 (0.11111111015256361)
#define NR_ATAN_Q8 (-0.14285714284666542)
#define NR_ATAN_Q9 (0.1999999999999552)
#define NR_ATAN_Q10 (-0.3333333333333333)

/* Quadrant/octant reduction, then atan(t) = pi/4 + atan((t-1)/(t+1)) above
 * tan(pi/8), then the polynomial; pi/4, pi/2 and pi are added as two-part
 * constants.  About one ulp for finite non-zero arguments; (0,0) -> 0. */
NR_HD double atan2_canon(double y, double x) {
    const double ax = fabs(x), ay = fabs(y);
    const bool swap = ay > ax;
    const double num = swap ? ax : ay;
    const double den = swap ? ay : ax;
    const double t = den == 0.0 ? 0.0 : num / den;
    const bool red = t > 0.41421356237309503;
    const double u = red ? (t - 1.0) / (t + 1.0) : t;
    const double z = u * u;
    double q = NR_ATAN_Q0;
    q = fma(q, z, NR_ATAN_Q1);
    q = fma(q, z, NR_ATAN_Q2);
    q = fma(q, z, NR_ATAN_Q3);
    q = fma(q, z, NR_ATAN_Q4);
    q = fma(q, z, NR_ATAN_Q5);
    q = fma(q, z, NR_ATAN_Q6);
    q = fma(q, z, NR_ATAN_Q7);
    q = fma(q, z, NR_ATAN_Q8);
    q = fma(q, z, NR_ATAN_Q9);
    q = fma(q, z, NR_ATAN_Q10);
    double r = fma(u * z, q, u);
    if (red) r = 0.7853981633974483 + (3.061616997868383e-17 + r);
    if (swap) r = 1.5707963267948966 + (6.123233995736766e-17 - r);
    if (x < 0.0) r = 3.141592653589793 + (1.2246467991473532e-16 - r);
    return y < 0.0 ? -r : r;
}

/* Periodic image offset wrap * width; exactly 0.0 for wrap 0. */
NR_HD double wrap_shift(int wrap, double width) { return wrap ? (double)wrap * width : 0.0; }

/* Stretch force on the bond's SECOND end's partner, i.e. the value the
 * reference adds to its first endpoint (large_strain_relax.cu:401-403);
 * the second endpoint receives the negation. */
NR_HD void bond_force(double x1, double y1, double x2, double y2, double wW, double l0, double k, double &fx,
                      double &fy) {
    const double rx = (x1 - x2) - wW, ry = y1 - y2;
    const double inv = 1.0 / sqrt(fma(rx, rx, ry * ry));
    const double s = k * fma(-l0, inv, 1.0);
    fx = s * ((x2 + wW) - x1);
    fy = s * (y2 - y1);
}

NR_HD double bond_energy(double x1, double y1, double x2, double y2, double wW, double l0, double k) {
    const double rx = (x1 - x2) - wW, ry = y1 - y2;
    const double dd = sqrt(fma(rx, rx, ry * ry)) - l0;
    return ((0.5 * k) * dd) * dd;
}

/* theta - theta0 for arms a = r_hj, b = r_hk; phi0 = theta0 - pi. */
NR_HD double bend_dtheta(double ax, double ay, double bx, double by, double phi0) {
    const double c = fma(ax, by, -(ay * bx));
    const double d = fma(ax, bx, ay * by);
    return atan2_canon(-c, -d) - phi0;
}

/* Bending forces on j and k (large_strain_relax.cu:453-459); the hinge
 * receives (-fjx - fkx, -fjy - fky). */
NR_HD void bend_force(double ax, double ay, double bx, double by, double kb, double phi0, double &fjx,
                      double &fjy, double &fkx, double &fky) {
    const double g = kb * bend_dtheta(ax, ay, bx, by, phi0);
    const double g2 = g / fma(ax, ax, ay * ay);
    const double g3 = g / fma(bx, bx, by * by);
    fjx = -ay * g2;
    fjy = ax * g2;
    fkx = by * g3;
    fky = -bx * g3;
}

NR_HD double bend_energy(double ax, double ay, double bx, double by, double kb, double phi0) {
    const double dth = bend_dtheta(ax, ay, bx, by, phi0);
    return ((0.5 * kb) * dth) * dth;
}

/* Virial of one bond, W = -sum over its two nodes of r_n (x) F_n with the
 * minimum-image vector r = r_j - r_i and the force f on i (j gets -f):
 * W_ab = r_a f_b.  Summed over bonds and triples and divided by the area,
 * W_xy is the shear stress sigma_xy = (1/A) dE/dgamma under the affine map
 * x += gamma (y - miny) that affine_displace applies
 * (large_strain_relax.cu:527-537), W_yy the normal stress under y +=
 * eps (y - miny), W_xx under x += eps x (the x period scaled with it). */
NR_HD void bond_virial(double x1, double y1, double x2, double y2, double wW, double l0, double k, double &wxx,
                       double &wyy, double &wxy) {
    double fx, fy;
    bond_force(x1, y1, x2, y2, wW, l0, k, fx, fy);
    const double rx = (x2 + wW) - x1, ry = y2 - y1;
    wxx = rx * fx;
    wyy = ry * fy;
    wxy = ry * fx;
}

/* Virial of one bending triple with arms a = r_hj, b = r_hk:
 * W_ab = -(a_a F_j,b + b_a F_k,b) (the hinge's -(F_j + F_k) sits at the
 * origin of the arms). */
NR_HD void bend_virial(double ax, double ay, double bx, double by, double kb, double phi0, double &wxx, double &wyy,
                       double &wxy) {
    double fjx, fjy, fkx, fky;
    bend_force(ax, ay, bx, by, kb, phi0, fjx, fjy, fkx, fky);
    wxx = -fma(ax, fjx, bx * fkx);
    wyy = -fma(ay, fjy, by * fky);
    wxy = -fma(ay, fjx, by * fkx);
}

/* Per-node reduction terms of the FIRE loop. */
NR_HD double dot2(double ax, double ay, double bx, double by) { return fma(ax, bx, ay * by); }

}  // namespace nr

#endif
