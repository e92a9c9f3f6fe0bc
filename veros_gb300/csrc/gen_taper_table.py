"""Generate taper_table.inc: piecewise Taylor coefficients of the slope taper.

The taper of veros/core/isoneutral/isoneutral.py:10-15 is
f(x) = 0.5 * (1 + tanh(x)) with x = (iso_slopec - |s|) / iso_dslope. For
the centres c_n = X0 + n/256, n = 0..(X1-X0)*256, the table holds the Taylor
coefficients f^(k)(c_n)/k!, k = 0..4, computed with mpmath at 40 significant
digits and rounded to double, followed by c_n itself; entry n serves |x - c_n| <= 1/512, so the table
covers [X0 - 1/512, X1 + 1/512). The truncation error is below 2e-15
(max |f^(5)| < 8 on the range, (1/512)^5 / 5!), 1e-15 of the taper's range
and far below the 1e-12 bar of the outputs. Centres on the 1/256 grid let
the kernel find n by rounding x*256 to the nearest integer.

Run from the repository root: python veros_gb300/csrc/gen_taper_table.py
"""

import os

import mpmath as mp

X0, X1, PER_UNIT, DEG = -4, 2, 256, 4


def main():
    mp.mp.dps = 40
    n = (X1 - X0) * PER_UNIT + 1
    f = lambda x: mp.mpf("0.5") * (1 + mp.tanh(x))  # noqa: E731
    rows = []
    for i in range(n):
        c = mp.mpf(X0) + mp.mpf(i) / PER_UNIT
        coef = mp.taylor(f, c, DEG) + [c]  # the row's centre last
        rows.append("  {" + ", ".join(repr(float(v)) for v in coef) + "},")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "taper_table.inc")
    with open(out, "w") as fh:
        fh.write("// Generated by gen_taper_table.py: Taylor coefficients (degree %d) of\n" % DEG)
        fh.write("// 0.5*(1+tanh(x)) about the centres %d + n/%d, n = 0..%d.\n" % (X0, PER_UNIT, n - 1))
        fh.write("constexpr double kTaperX0 = %d.0;\n" % X0)
        fh.write("constexpr double kTaperX1 = %d.0;\n" % X1)
        fh.write("constexpr double kTaperPerUnit = %d.0;\n" % PER_UNIT)
        fh.write("constexpr int kTaperN = %d;\n" % n)
        fh.write("constexpr int kTaperDeg = %d;\n" % DEG)
        fh.write("// row n: f^(k)(c_n)/k! for k = 0..%d, then c_n\n" % DEG)
        fh.write("static __device__ const double kTaperCoef[%d][%d] = {\n" % (n, DEG + 2))
        fh.write("\n".join(rows))
        fh.write("\n};\n")
    print(out)


if __name__ == "__main__":
    main()
