"""Coefficients of the polynomial forms of the logarithmic mean used by the
device code (tag_common.cuh).

With f = ((y - x)/(y + x))^2 and z = sqrt(f),
    ln_mean(x, y)     = (x + y)/2 * R(f),   R(f) = z / atanh(z),
    inv_ln_mean(x, y) = 2/(x + y) * Q(f),   Q(f) = atanh(z) / z = sum_k f^k/(2k+1).
On an interval [0, F] each function is written as 1 + f * s(f) with s a
polynomial of degree m - 1: the Chebyshev interpolant of s = (R - 1)/f (or
(Q - 1)/f) at m Chebyshev points of [0, F], converted to monomials and rounded
to double (Chebyshev economization of the Taylor series, C. Lanczos, J. Math.
Phys. 17 (1938) 123-199).  It reaches the same accuracy as the Taylor series
with fewer terms: for F = 0.09 nine (R) and ten (Q) coefficients instead of
sixteen, for F = 0.01 six instead of eight.

Run as a script to print the C++ coefficient lists and the maximum relative
error of each rounded polynomial over its interval (50-digit arithmetic)."""
import mpmath as mp

mp.mp.dps = 50

# (name, function, interval end F, number of coefficients after the leading 1)
FORMS = (
    ("R", "R", "0.09", 9),
    ("Q", "Q", "0.09", 10),
    ("R", "R", "0.01", 6),
    ("Q", "Q", "0.01", 6),
)


def exact(fun, f):
    f = mp.mpf(f)
    if f == 0:
        return mp.mpf(1)
    z = mp.sqrt(f)
    return z / mp.atanh(z) if fun == "R" else mp.atanh(z) / z


def tail(fun, f):
    """s(f) = (R(f) - 1)/f or (Q(f) - 1)/f, with its limit at f = 0."""
    f = mp.mpf(f)
    if f == 0:
        return mp.mpf(-1) / 3 if fun == "R" else mp.mpf(1) / 3
    return (exact(fun, f) - 1) / f


def coefficients(fun, F, m):
    """Monomial coefficients c[0..m-1] of the degree m-1 Chebyshev interpolant of
    s on [0, F]; the form is 1 + f (c0 + f (c1 + ...))."""
    F = mp.mpf(F)
    nodes = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / m) for k in range(m)]
    vals = [tail(fun, F / 2 * (t + 1)) for t in nodes]
    cheb = [2 * mp.fsum(vals[k] * mp.cos(mp.pi * j * (k + mp.mpf(1) / 2) / m) for k in range(m)) / m
            for j in range(m)]
    cheb[0] /= 2
    # T_j(t) with t = 2 f / F - 1, as polynomials in f
    a, b = 2 / F, mp.mpf(-1)
    T = [[mp.mpf(1)], [b, a]]
    for j in range(2, m):
        nxt = [mp.mpf(0)] * (j + 1)
        for i, v in enumerate(T[j - 1]):
            nxt[i] += 2 * b * v
            nxt[i + 1] += 2 * a * v
        for i, v in enumerate(T[j - 2]):
            nxt[i] -= v
        T.append(nxt)
    mono = [mp.mpf(0)] * m
    for j in range(m):
        for i, v in enumerate(T[j]):
            mono[i] += cheb[j] * v
    return [float(c) for c in mono]


def max_rel_error(fun, F, coefs, samples=2000):
    """Maximum over [0, F] of |p(f)/fun(f) - 1| for p = 1 + f (c0 + f (c1 + ...))
    with the double coefficients evaluated exactly."""
    F = mp.mpf(F)
    worst = mp.mpf(0)
    for k in range(samples + 1):
        f = F * k / samples
        p = mp.mpf(0)
        for c in reversed(coefs):
            p = p * f + mp.mpf(c)
        p = 1 + f * p
        worst = max(worst, abs(p / exact(fun, f) - 1))
    return worst


if __name__ == "__main__":
    for name, fun, F, m in FORMS:
        c = coefficients(fun, F, m)
        print(f"// {name} on [0, {F}], {m} coefficients, max rel. error "
              f"{mp.nstr(max_rel_error(fun, F, c), 3)}")
        print("{" + ", ".join(repr(v) for v in c) + "}")
