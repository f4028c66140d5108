"""The integer threshold test of the selection and scoring kernels
(RatioAtLeast / SplitThreshold in beam_gb300/csrc/merge.cu), restated step
for step in Python and checked against the reference's double test
RN(gain / before) >= threshold (Python floats are IEEE doubles) at and around
the boundary: thresholds 1/(iter+1) split into m * 2^-e, exact multiples of
the threshold's rational value, and gains one below and above them.

The GPU golden tests run the kernels themselves on every fixture; this test
pins the method's argument (monotonic rounding, the 2^-51 band) on the CPU."""

import math
import random


def split(threshold):
    if threshold > 0 and math.isfinite(threshold):
        f, ex = math.frexp(threshold)  # threshold = f * 2^ex, f in [0.5, 1)
        return int(math.ldexp(f, 53)), 53 - ex
    return 0, -1


def ratio_at_least(gain, before, threshold, t):
    m, e = t
    if 0 <= e <= 63 and gain < (1 << 53) and before < (1 << 53):
        lhs = gain << e
        rhs = m * before
        if lhs >= rhs:
            return True
        if lhs + (rhs >> 51) < rhs:
            return False
    return gain / before >= threshold


def test_split_is_exact():
    for it in range(1, 1000):
        th = 1.0 / (it + 1)
        m, e = split(th)
        assert m < (1 << 53) and m * 2.0 ** -e == th


def test_integer_test_matches_the_double_test():
    rng = random.Random(5)
    cases = 0
    for it in list(range(1, 60)) + [99, 255, 1023, 4095]:
        th = 1.0 / (it + 1)
        t = split(th)
        # exact multiples of 1/(it+1) and their neighbours
        for k in (1, 3, 7, 12345, 10**9, (1 << 40) + 1):
            b = k * (it + 1)
            if b >= 1 << 53:
                continue
            for g in (k - 1, k, k + 1):
                if g > 0:
                    assert ratio_at_least(g, b, th, t) == (g / b >= th)
                    cases += 1
        # random denominators of every scale, gains next to the boundary
        for _ in range(600):
            b = rng.choice([rng.randint(1, 100), rng.randint(1, 10**6), rng.randint(1, 10**15),
                            rng.randint(1, (1 << 53) - 1)])
            g0 = int(b * th)
            for g in (g0 - 1, g0, g0 + 1, rng.randint(1, 2 * b + 1)):
                if g > 0:
                    assert ratio_at_least(g, b, th, t) == (g / b >= th)
                    cases += 1
    assert cases > 100000
