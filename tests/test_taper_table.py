"""The taper table of the slope kernel (csrc/taper_table.inc) against the
taper 0.5 * (1 + tanh(x)) of veros/core/isoneutral/isoneutral.py:10-15.

The kernel picks entry n = round(P (x - X0)) (P entries per unit) from the
low word of x*P + (1.5*2^52 - P*X0) and evaluates the entry's Taylor
polynomial at b = x - c_n, c_n = X0 + n/P stored at the end of the row.
This restates that arithmetic in NumPy (the product x*P is exact for a
power-of-two P, so a plain add rounds like the kernel's fused multiply-add) and checks the result against mpmath on
random arguments and on both edges of every interval, within the table's
truncation bound.
"""

import os
import re
import struct

import numpy as np
import pytest

INC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "veros_gb300", "csrc",
                   "taper_table.inc")
MAGIC = 6755399441055744.0  # 1.5 * 2^52


def _table():
    txt = open(INC).read()
    x0 = float(re.search(r"kTaperX0 = (-?[\d.]+)", txt).group(1))
    per = float(re.search(r"kTaperPerUnit = ([\d.]+)", txt).group(1))
    n = int(re.search(r"kTaperN = (\d+)", txt).group(1))
    deg = int(re.search(r"kTaperDeg = (\d+)", txt).group(1))
    rows = re.findall(r"\{([^{}]+)\},", txt.split("kTaperCoef")[1])
    table = np.array([[float(v) for v in r.split(",")] for r in rows])
    assert table.shape == (n, deg + 2)
    assert np.array_equal(table[:, deg + 1], x0 + np.arange(n) / per)  # each row's centre
    return x0, per, table


def _taper_table(x, x0, per, coef):
    y = np.float64(x) * per + (MAGIC - x0 * per)
    bits = struct.unpack("<Q", struct.pack("<d", y))[0]
    lo, hi = np.int64(np.uint32(bits & 0xFFFFFFFF)).astype(np.int32), bits >> 32
    if hi != 0x43380000 or not 0 <= lo < coef.shape[0]:
        return None
    deg = coef.shape[1] - 2
    b = x - coef[lo, deg + 1]
    r = coef[lo, deg]
    for k in range(deg - 1, -1, -1):
        r = r * b + coef[lo, k]
    return r


def test_table_matches_the_taper_to_rounding():
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 30
    x0, per, coef = _table()
    n = coef.shape[0]
    centres = x0 + np.arange(n) / per
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(x0, x0 + (n - 1) / per, 4000), centres[::4] + 0.5 / per - 1e-14,
                         centres[::4] - 0.5 / per + 1e-14])
    worst = 0.0
    for x in xs:
        t = _taper_table(float(x), x0, per, coef)
        assert t is not None, x
        ref = float(mp.mpf("0.5") * (1 + mp.tanh(mp.mpf(float(x)))))
        worst = max(worst, abs(t - ref))
    # truncation bound of the table: max |f^(deg+1)| (1/(2P))^(deg+1) / (deg+1)! (2e-15 for degree 4 at
    # P = 256) plus the polynomial's own rounding
    assert worst <= 2.5e-15, worst


def test_out_of_table_arguments_take_the_tail_path():
    x0, per, coef = _table()
    n = coef.shape[0]
    for x in (x0 - 0.6 / per, x0 + (n - 1) / per + 0.6 / per, -50.0, 50.0, float("inf"), float("-inf"),
              float("nan")):
        assert _taper_table(x, x0, per, coef) is None, x
