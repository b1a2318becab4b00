"""The ensemble's active-set window (exact::active_window in
gravidy_gb300/csrc/h4_exact.cuh) restated with exact rational arithmetic and
checked against the reference's test itself: a particle is active when
|itime - (t + dt)| < 2^-51 in IEEE double arithmetic
(Hermite4::find_particles_to_move, Hermite4.cpp:64-88).  The window [lo, hi]
is formed from itime - 2^-51 rounded up and itime + 2^-51 rounded down, each
moved one ulp inward when exact; for itime >= 2^-48 it must hold exactly the
tn that pass.  The device code forms the same bounds with __dadd_ru /
__dadd_rd; the GPU tests check its active sets bit for bit against the oracle.
"""
import math
import random
import struct
from fractions import Fraction

E = 2.0 ** -51


def bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def round_up(q):
    x = float(q)                      # nearest
    return x if Fraction(x) >= q else math.nextafter(x, math.inf)


def round_down(q):
    x = float(q)
    return x if Fraction(x) <= q else math.nextafter(x, -math.inf)


def window(itime):
    a = round_up(Fraction(itime) - Fraction(E))
    if Fraction(a) == Fraction(itime) - Fraction(E):
        a = math.nextafter(a, math.inf)
    b = round_down(Fraction(itime) + Fraction(E))
    if Fraction(b) == Fraction(itime) + Fraction(E):
        b = math.nextafter(b, -math.inf)
    return bits(a), bits(b)


def reference_active(itime, tn):
    return abs(itime - tn) < E        # IEEE double subtraction, as the reference


def candidates(itime, rng):
    out = [itime, 0.0, itime * 2, itime / 2, math.inf]
    x = y = itime
    for _ in range(40):               # neighbours in ulps, across binade edges
        x = math.nextafter(x, math.inf)
        y = math.nextafter(y, -math.inf)
        out += [x, y]
    for _ in range(20):               # within a few 2^-51 of itime
        out.append(itime + rng.uniform(-3, 3) * E)
    return [t for t in out if t >= 0.0]


def test_window_holds_exactly_the_active_tn():
    rng = random.Random(7)
    times = [2.0 ** -k for k in range(0, 48)] + [3 * 2.0 ** -k for k in range(1, 46)]
    times += [k * 2.0 ** -23 for k in (1, 3, 5, 1023, 1025, 2 ** 20 - 1, 2 ** 20 + 1)]
    times += [rng.uniform(2.0 ** -48, 8.0) for _ in range(200)]
    times += [1.0, 2.0, 4.0, 0.125, 0.0625 + 2.0 ** -23]
    checked = 0
    for itime in times:
        assert itime >= 2.0 ** -48
        lo, hi = window(itime)
        for tn in candidates(itime, rng):
            assert (lo <= bits(tn) <= hi) == reference_active(itime, tn), (itime.hex(), tn.hex())
            checked += 1
    assert checked > 30000


def test_window_brackets_itime_and_stays_narrow():
    for itime in (2.0 ** -48, 2.0 ** -23, 0.5, 1.0, 1.5, 2.0, 3.0, 7.99):
        lo, hi = window(itime)
        assert lo <= bits(itime) <= hi
        # 2^-51 / ulp(itime) patterns above, at most twice that below (the
        # binade below a power of two has half the ulp)
        assert hi - lo <= 3 * max(1.0, E / math.ulp(itime)) + 2
