"""The integer-path binary64 operations (csrc/fp64_emu.cuh, compiled for
the host) against exact rational arithmetic: each result must be the
binary64 number that rounding the exact sum or product down, up or to
nearest (ties to even) gives.  The operands are chosen edge cases: ties,
carries into the next binade, the edges of the normal range, far and close
exponents and near-cancellation, plus structured random pairs.  No GPU and
no FPU rounding mode is involved."""

from __future__ import annotations

import ctypes as C
import math
import random
from fractions import Fraction

import pytest

from cuminlp_gb300._lib import check, lib

MIN_NORMAL = 2.0 ** -1022
ULP1 = 2.0 ** -52


@pytest.fixture(scope="module", autouse=True)
def _built():
    from cuminlp_gb300 import build
    build.build_library()


def exact(op: int, a: float, b: float) -> Fraction:
    fa, fb = Fraction(a), Fraction(b)
    return fa + fb if op < 2 else fa - fb if op < 4 else fa * fb


def rounded(q: Fraction, op: int) -> float:
    """q rounded to binary64: down (even op), up (odd op below 6), or to
    nearest with ties to even (op 6; int / int division in Python rounds
    correctly)."""
    x = q.numerator / q.denominator
    if op == 6:
        return x
    if op % 2 == 0:
        return x if Fraction(x) <= q else math.nextafter(x, -math.inf)
    return x if Fraction(x) >= q else math.nextafter(x, math.inf)


def emu(op: int, a: float, b: float):
    out = C.c_double()
    handled = C.c_int32()
    check(lib().cmn_fp64_emu_op_host(op, a, b, C.byref(out), C.byref(handled)))
    return bool(handled.value), out.value


def edge_pairs():
    one_up = 1.0 + ULP1
    big = 2.0 - ULP1
    pairs = [
        (one_up, 1.5), (1.0 + 3 * ULP1, 1.5), (one_up, one_up), (big, big), (big, 1.0 + ULP1),
        (1.0, 2.0 ** -60), (1.0, -(2.0 ** -60)), (1.0, -(1.0 - 2.0 ** -53)), (one_up, -1.0),
        (2.0 ** -511, 2.0 ** -511), (2.0 ** -511 * one_up, 2.0 ** -511), (MIN_NORMAL, 1.0 + ULP1),
        (MIN_NORMAL * 3, -MIN_NORMAL), (2.0 ** 511 * big, 2.0 ** 511), (1.7976931348623157e308, 0.5),
        (-3.0, 1.0 / 3.0), (0.1, 0.2), (-0.1, 0.3), (1e300, 1e-300), (math.pi, -math.e),
        (123456789.0, 1.0 / 123456789.0), (-(2.0 ** 1023), -1.5),
    ]
    # products whose dropped bits are exactly one half: ties for rounding to nearest
    for k in range(1, 40, 2):
        pairs.append((1.0 + k * ULP1, 1.5))
        pairs.append((-(1.0 + k * ULP1), 1.5))
        pairs.append((1.0 + k * ULP1, 3.0))
    return pairs


def random_pairs(n: int, seed: int):
    rng = random.Random(seed)
    out = []
    for _ in range(n):
        ea = rng.randint(-40, 40)
        eb = ea + rng.choice([0, 0, 1, -1, 2, rng.randint(-60, 60)])
        ma = 1.0 + rng.getrandbits(52) * ULP1
        mb = 1.0 + rng.choice([rng.getrandbits(52), (1 << 52) - 1, 1, 0, rng.getrandbits(8)]) * ULP1
        a = math.ldexp(ma, ea) * rng.choice([1, -1])
        b = math.ldexp(mb, eb) * rng.choice([1, -1])
        if rng.random() < 0.1:  # near-cancellation
            b = -math.nextafter(a, rng.choice([math.inf, -math.inf]))
        out.append((a, b))
    return out


@pytest.mark.parametrize("source", ["edges", "random"])
def test_integer_path_is_exactly_rounded(source):
    pairs = edge_pairs() if source == "edges" else random_pairs(4000, 17)
    handled = bad = 0
    for a, b in pairs:
        for op in range(7):
            ok, got = emu(op, a, b)
            if not ok:
                continue
            handled += 1
            want = rounded(exact(op, a, b), op)
            if got != want or math.copysign(1.0, got) != math.copysign(1.0, want):
                bad += 1
                assert bad < 5, (op, a.hex(), b.hex(), got.hex(), want.hex())
    assert bad == 0
    assert handled > len(pairs) * 5  # nearly every pair stays on the integer path


def test_non_normal_operands_fall_back():
    for a, b in ((0.0, 1.0), (5e-324, 1.0), (math.inf, 1.0), (math.nan, 2.0), (1.0, -1.0)):
        ok, _ = emu(0, a, b)
        assert not ok, (a, b)
    ok, _ = emu(4, MIN_NORMAL, 0.5)  # a subnormal product
    assert not ok
    ok, _ = emu(5, 1.7976931348623157e308, 2.0)  # overflow
    assert not ok
