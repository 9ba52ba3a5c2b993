"""Generate ias15_constants.h: Gauss-Radau spacings and the g<->b transforms of
the 15th-order IAS15 integrator (Rein & Spiegel 2015, MNRAS 446, 1424).

The 8 spacings h_0 = 0 < h_1 < ... < h_7 < 1 are the Gauss-Radau nodes on
[0, 1] with the left end fixed: h = (1 + x)/2 for x = -1 and the 7 roots of
(P_7(x) + P_8(x))/(1 + x), P_n the Legendre polynomials.  The acceleration
over a step is a(h) = a_0 + sum_k b_k h^(k+1) (monomial form) or, in Newton
form, a(h) = a_0 + sum_j g_j h prod_{i=1..j} (h - h_i).  C maps g -> b
(b_k = sum_j C[j][k] g_j) and D = C^-1 maps b -> g.  Everything is computed
with 50 significant digits and rounded once to double.

Run:  python gen_ias15_constants.py > ias15_constants.h
"""
import mpmath as mp

mp.mp.dps = 50


def legendre_coeffs(n):
    """Coefficients (lowest degree first) of P_n by Bonnet's recurrence."""
    p0, p1 = [mp.mpf(1)], [mp.mpf(0), mp.mpf(1)]
    if n == 0:
        return p0
    for k in range(1, n):
        nxt = [mp.mpf(0)] * (k + 2)
        for d, c in enumerate(p1):
            nxt[d + 1] += (2 * k + 1) * c / (k + 1)
        for d, c in enumerate(p0):
            nxt[d] -= k * c / (k + 1)
        p0, p1 = p1, nxt
    return p1


def radau_nodes():
    a, b = legendre_coeffs(7), legendre_coeffs(8)
    s = [(a[d] if d < len(a) else 0) + b[d] for d in range(9)]
    # divide by (1 + x): synthetic division at x = -1, highest degree first
    hi = list(reversed(s))
    q = [hi[0]]
    for c in hi[1:-1]:
        q.append(c - q[-1])
    assert abs(hi[-1] - q[-1]) < mp.mpf(10) ** -40      # remainder vanishes
    roots = sorted(mp.re(r) for r in mp.polyroots(q, maxsteps=200, extraprec=200))
    assert len(roots) == 7
    return [mp.mpf(0)] + [(1 + r) / 2 for r in roots]


def transforms(h):
    # C[j][k]: coefficient of h^(k+1) in h * prod_{i=1..j} (h - h_i)
    C = [[mp.mpf(0)] * 7 for _ in range(7)]
    for j in range(7):
        poly = [mp.mpf(1)]            # coefficients of prod (h - h_i), lowest degree first
        for i in range(1, j + 1):
            new = [mp.mpf(0)] * (len(poly) + 1)
            for d, c in enumerate(poly):
                new[d + 1] += c
                new[d] -= c * h[i]
            poly = new
        for d, c in enumerate(poly):
            C[j][d] = c
    M = mp.matrix(7, 7)
    for j in range(7):
        for k in range(7):
            M[k, j] = C[j][k]          # b = M g
    Dm = M ** -1                       # g = Dm b
    D = [[Dm[j, k] for k in range(7)] for j in range(7)]
    return C, D


def main():
    h = radau_nodes()
    C, D = transforms(h)
    fmt = lambda v: mp.nstr(v, 21, min_fixed=-1, max_fixed=1) if v != 0 else "0.0"
    out = []
    out.append("/* Generated by gen_ias15_constants.py -- do not edit. */")
    out.append("#ifndef ASSIST_GB300_IAS15_CONSTANTS_H")
    out.append("#define ASSIST_GB300_IAS15_CONSTANTS_H")
    out.append("/* Gauss-Radau spacings on [0,1], h[0] = 0. */")
    out.append("#define IAS15_H_INIT { " + ", ".join(fmt(v) for v in h) + " }")
    out.append("/* RR(n,j) = h[n] - h[j] for 1 <= n <= 7, 0 <= j < n, row-major by n. */")
    rr = [h[n] - h[j] for n in range(1, 8) for j in range(n)]
    out.append("#define IAS15_RR_INIT { " + ", ".join(fmt(v) for v in rr) + " }")
    out.append("/* Inverse of RR, same order (divisions become multiplications). */")
    out.append("#define IAS15_RRINV_INIT { " + ", ".join(fmt(1 / v) for v in rr) + " }")
    out.append("/* C[j][k] for k < j: b_k += C[j][k] * (change of g_j); C[j][j] = 1. Row-major j = 1..6, k = 0..j-1. */")
    cc = [C[j][k] for j in range(1, 7) for k in range(j)]
    out.append("#define IAS15_C_INIT { " + ", ".join(fmt(v) for v in cc) + " }")
    out.append("/* D[j][k] for k > j: g_j = b_j + sum_k D[j][k] b_k. Row-major j = 0..5, k = j+1..6. */")
    dd_ = [D[j][k] for j in range(6) for k in range(j + 1, 7)]
    out.append("#define IAS15_D_INIT { " + ", ".join(fmt(v) for v in dd_) + " }")
    out.append("#endif")
    print("\n".join(out))


if __name__ == "__main__":
    main()
