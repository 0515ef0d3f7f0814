"""Generate ellint_coeffs.h: the coefficient tables of Fukushima's piecewise
Taylor method for the complete elliptic integrals K(m) and E(m)
(T. Fukushima, "Fast computation of complete elliptic integrals and Jacobian
elliptic functions", Celest. Mech. Dyn. Astr. 105 (2009) 305-328).

The reference evaluates this method in src/wlcs.c:460-809 (function
``ellint``).  The tables are not transcribed from it: every coefficient is
recomputed here from the mathematics with mpmath at 50 digits,

* K_j, E_j : Taylor coefficients K^(j)(m0)/j!, E^(j)(m0)/j! about the
  interval centres m0 = 0.05, 0.15, ..., 0.75, 0.825, 0.875, with the same
  number of terms per interval as the reference;
* q_j      : coefficients of the nome series q(m) = sum_j q_j m^j (exact
  dyadic rationals, j = 1..14);
* H_j      : Taylor coefficients of K(m) - E(m) about m = 0.05 (j = 0..10),
  used with Legendre's relation for m >= 0.9.

One deliberate deviation reproduces the reference: its 20th K coefficient of
the m0 = 0.875 interval is ten times the Taylor value (src/wlcs.c:728).  The
bug-compatible evaluator uses that value; the corrected evaluator uses the
Taylor value.  Run: ``python gen_ellint_coeffs.py`` (writes the header next
to this file).
"""
import os

import mpmath as mp

mp.mp.dps = 50

# (centre, number of K terms, number of E terms) per interval, as in the
# reference's switch cases 0..9.
INTERVALS = [
    (0.05, 11, 10), (0.15, 12, 11), (0.25, 12, 11), (0.35, 13, 12),
    (0.45, 14, 13), (0.55, 15, 13), (0.65, 17, 15), (0.75, 20, 17),
    (0.825, 16, 14), (0.875, 20, 17),
]
NK_MAX = 20
NE_MAX = 17


def dbl(x):
    return repr(float(x))


def main():
    ktab, etab = [], []
    for m0, nk, ne in INTERVALS:
        tk = mp.taylor(mp.ellipk, mp.mpf(str(m0)), nk - 1)
        te = mp.taylor(mp.ellipe, mp.mpf(str(m0)), ne - 1)
        ktab.append([tk[j] for j in range(nk)] + [0] * (NK_MAX - nk))
        etab.append([te[j] for j in range(ne)] + [0] * (NE_MAX - ne))
    # reference deviation: interval 9 (m0 = 0.875), K term 19 is 10x.
    kref9_19 = ktab[9][19] * 10
    qn = mp.taylor(lambda m: mp.qfrom(m=m), 0, 14)
    hn = mp.taylor(lambda m: mp.ellipk(m) - mp.ellipe(m), mp.mpf("0.05"), 10)

    out = []
    w = out.append
    w("/* Generated by gen_ellint_coeffs.py -- do not edit.  Coefficients of")
    w(" * Fukushima's piecewise Taylor method for K(m), E(m) (Celest. Mech. Dyn.")
    w(" * Astr. 105 (2009) 305-328), recomputed with mpmath at 50 digits.  Shared")
    w(" * by host and device code: the includer defines TP_ELL_QUAL (e.g.")
    w(" * `static const` or `__constant__ static const`). */")
    w("#ifndef TP_ELL_QUAL")
    w("#define TP_ELL_QUAL static const")
    w("#endif")
    w("#define TP_ELL_NCASE 10")
    w("#define TP_ELL_NK_MAX %d" % NK_MAX)
    w("#define TP_ELL_NE_MAX %d" % NE_MAX)
    w("TP_ELL_QUAL double tp_ell_m0[TP_ELL_NCASE] = {%s};" %
      ", ".join(dbl(m0) for m0, _, _ in INTERVALS))
    w("TP_ELL_QUAL int tp_ell_nk[TP_ELL_NCASE] = {%s};" %
      ", ".join(str(nk) for _, nk, _ in INTERVALS))
    w("TP_ELL_QUAL int tp_ell_ne[TP_ELL_NCASE] = {%s};" %
      ", ".join(str(ne) for _, _, ne in INTERVALS))
    w("TP_ELL_QUAL double tp_ell_k[TP_ELL_NCASE][TP_ELL_NK_MAX] = {")
    for row in ktab:
        w("  {%s}," % ", ".join(dbl(c) for c in row))
    w("};")
    w("TP_ELL_QUAL double tp_ell_e[TP_ELL_NCASE][TP_ELL_NE_MAX] = {")
    for row in etab:
        w("  {%s}," % ", ".join(dbl(c) for c in row))
    w("};")
    w("/* The reference's value of K term 19 of the m0 = 0.875 interval (10x the")
    w(" * Taylor coefficient); used only by the bug-compatible evaluator. */")
    w("#define TP_ELL_K9_19_REF %s" % dbl(kref9_19))
    w("/* nome series q(m) = sum_{j=1}^{14} q_j m^j; entry 0 unused */")
    w("TP_ELL_QUAL double tp_ell_q[15] = {%s};" % ", ".join(dbl(c) for c in qn))
    w("/* Taylor coefficients of K(m) - E(m) about m = 0.05 */")
    w("TP_ELL_QUAL double tp_ell_h[11] = {%s};" % ", ".join(dbl(c) for c in hn))
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ellint_coeffs.h")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
