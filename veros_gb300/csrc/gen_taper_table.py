"""Generate taper_table.inc: piecewise Taylor coefficients of the slope taper.

The taper of veros/core/isoneutral/isoneutral.py:10-15 is
f(x) = 0.5 * (1 + tanh(x)) with x = (iso_slopec - |s|) / iso_dslope. On
[X0, X1) the table holds, for intervals of width 1/64, the Taylor
coefficients f^(n)(c)/n!, n = 0..6, about each interval centre c, computed
with mpmath at 40 significant digits and rounded to double. With |x - c| <=
1/128 the truncation error is below 5e-17 (max |f^(7)| = 136 on the range).

Run from the repository root: python veros_gb300/csrc/gen_taper_table.py
"""

import os

import mpmath as mp

X0, X1, PER_UNIT, DEG = -4, 2, 64, 6


def main():
    mp.mp.dps = 40
    n = (X1 - X0) * PER_UNIT
    f = lambda x: mp.mpf("0.5") * (1 + mp.tanh(x))  # noqa: E731
    rows = []
    for i in range(n):
        c = mp.mpf(X0) + (mp.mpf(i) + mp.mpf("0.5")) / PER_UNIT
        coef = mp.taylor(f, c, DEG)
        rows.append("  {" + ", ".join(repr(float(v)) for v in coef) + "},")
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "taper_table.inc")
    with open(out, "w") as fh:
        fh.write("// Generated by gen_taper_table.py: Taylor coefficients (degree %d) of\n" % DEG)
        fh.write("// 0.5*(1+tanh(x)) about the centres of 1/%d-wide intervals on [%d, %d).\n" % (PER_UNIT, X0, X1))
        fh.write("constexpr double kTaperX0 = %d.0;\n" % X0)
        fh.write("constexpr double kTaperX1 = %d.0;\n" % X1)
        fh.write("constexpr double kTaperPerUnit = %d.0;\n" % PER_UNIT)
        fh.write("constexpr int kTaperN = %d;\n" % n)
        fh.write("constexpr int kTaperDeg = %d;\n" % DEG)
        fh.write("static __device__ const double kTaperCoef[%d][%d] = {\n" % (n, DEG + 1))
        fh.write("\n".join(rows))
        fh.write("\n};\n")
    print(out)


if __name__ == "__main__":
    main()
