"""Derives the polynomial used by nr_canon_atan2 (canon_math.h) and its C twin
in the oracle.

Method: atan(u) = u + u*z*Q(z), z = u*u, on |u| <= tan(pi/8); the argument
reduction atan(t) = pi/4 + atan((t-1)/(t+1)) covers tan(pi/8) < t <= 1 and
atan(t) = pi/2 - atan(1/t) covers t > 1.  Q is the Chebyshev interpolant of
(atan(sqrt z)/sqrt z - 1)/z on [0, tan(pi/8)^2], computed in 60-digit
arithmetic with mpmath and converted to monomial form (Horner order, highest
power first).  Run it to reprint the table; it also reports the worst error of
the double-precision evaluation against mpmath on a dense grid.
"""
import mpmath as mp

mp.mp.dps = 60
DEG = 10
ZMAX = mp.tan(mp.pi / 8) ** 2


def q_exact(z):
    if z == 0:
        return mp.mpf(-1) / 3
    s = mp.sqrt(z)
    return (mp.atan(s) / s - 1) / z


def cheb_coeffs():
    n = DEG + 1
    nodes = [ZMAX / 2 * (1 + mp.cos(mp.pi * (k + mp.mpf(1) / 2) / n)) for k in range(n)]
    vals = [q_exact(z) for z in nodes]
    # Solve the Vandermonde system for monomial coefficients in 60 digits.
    A = mp.matrix([[z ** j for j in range(n)] for z in nodes])
    c = mp.lu_solve(A, mp.matrix(vals))
    return [c[j] for j in range(n)]


def fma(a, b, c):
    """Correctly rounded a*b + c (the product is exact at 60 digits)."""
    return float(mp.mpf(a) * mp.mpf(b) + mp.mpf(c))


def atan_double(u, coeffs):
    z = u * u
    q = coeffs[-1]
    for c in reversed(coeffs[:-1]):
        q = fma(q, z, c)
    return fma(u * z, q, u)


if __name__ == "__main__":
    cs = cheb_coeffs()
    dcs = [float(c) for c in cs]
    worst = 0.0
    for i in range(1, 20001):
        u = float(mp.tan(mp.pi / 8)) * i / 20000
        got = atan_double(u, dcs)
        ref = mp.atan(mp.mpf(u))
        err = abs((mp.mpf(got) - ref) / ref) / 2.0 ** -53
        worst = max(worst, float(err))
    print("worst relative error on (0, tan(pi/8)]: %.3f half-ulps" % worst)
    for j in reversed(range(len(dcs))):
        print("    %s,  /* z^%d */" % (repr(dcs[j]), j))
