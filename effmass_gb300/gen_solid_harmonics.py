#!/usr/bin/env python3
"""Generate csrc/solid_harmonics.inc: the real solid harmonics R_lm(K) = |K|^l Y_lm(K^)
as homogeneous polynomials in (Kx, Ky, Kz), l <= 4, in the convention of the
reference's real spherical harmonics (src/math/sph_harmonics.cppm:702-735):
  Y_l0 = N_l0 P_l^0(cos t),  Y_{l,m>0} = sqrt(2) N_lm P_l^m(cos t) cos(m p),
  Y_{l,m<0} = sqrt(2) N_l|m| P_l^|m|(cos t) sin(|m| p),
  N_lm = sqrt((2l+1)/(4 pi) (l-m)!/(l+m)!),  P_l^m with the Condon-Shortley (-1)^m.
Rows are ordered by lm = l*l + l + m.  Run from the repository root:
    python effmass_gb300/gen_solid_harmonics.py
"""
import os

import sympy as sp

LMAX = 4
x, y, z, t = sp.symbols("x y z t", real=True)


def solid(l, m):
    am = abs(m)
    # P_l^m(t) = (-1)^m (1-t^2)^(m/2) d^m P_l / dt^m; (1-t^2)^(m/2) r^m = rho^m
    dP = sp.diff(sp.legendre(l, t), t, am)
    N = sp.sqrt(sp.Rational(2 * l + 1, 1) / (4 * sp.pi) * sp.factorial(l - am) / sp.factorial(l + am))
    r2 = x * x + y * y + z * z
    # r^(l-m) dP(z/r): dP has parity (l-m) so this is a polynomial in z and r^2
    poly = sp.expand(dP.subs(t, z))
    deg = l - am
    hom = 0
    for (k,), c in sp.Poly(poly, z).terms():
        hom += c * z ** k * r2 ** ((deg - k) // 2)
    if am == 0:
        ang = 1
    else:
        w = sp.expand((x + sp.I * y) ** am)
        ang = sp.sqrt(2) * (sp.re(w) if m > 0 else sp.im(w))
    R = sp.expand((-1) ** am * N * hom * ang)
    return sp.Poly(R, x, y, z)


def main():
    rows = []
    for l in range(LMAX + 1):
        for m in range(-l, l + 1):
            P = solid(l, m)
            terms = [(float(sp.N(c, 30)), a, b, cc) for (a, b, cc), c in P.terms() if c != 0]
            rows.append((l, m, terms))
    nt = max(len(r[2]) for r in rows)
    out = ["// Generated by effmass_gb300/gen_solid_harmonics.py: real solid harmonics",
           "// R_lm(K) = |K|^l Y_lm(K^) as sum_t c_t Kx^a Ky^b Kz^c, l <= %d, rows lm = l*l + l + m." % LMAX,
           "#define HPSI_SH_LMAX %d" % LMAX, "#define HPSI_SH_TERMS %d" % nt,
           "struct ShTerm { double c; int a, b, z; };",
           "__device__ __constant__ int kShCount[%d] = {%s};" % (len(rows), ", ".join(str(len(r[2])) for r in rows)),
           "__device__ __constant__ ShTerm kSh[%d][HPSI_SH_TERMS] = {" % len(rows)]
    for l, m, terms in rows:
        cells = ", ".join("{%.17g, %d, %d, %d}" % tt for tt in terms)
        pad = ", ".join(["{0.0, 0, 0, 0}"] * (nt - len(terms)))
        body = cells + (", " + pad if pad else "")
        out.append("    {%s},  // l=%d m=%d" % (body, l, m))
    out.append("};")
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "csrc", "solid_harmonics.inc"), "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
