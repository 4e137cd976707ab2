"""Seeded inputs for the field-file reader tests: number tokens that stress
correct rounding (exact decimal midpoints between adjacent doubles, cut and
nudged; subnormal and overflow edges; 20..900-digit mantissas) and the
float() grammar (signs, inf/nan spellings, underscores, whitespace, malformed
forms), plus whole CSV texts in the savetxt layout of the reference's files."""
from __future__ import annotations

import random
import struct
from decimal import Decimal, getcontext
from fractions import Fraction

import numpy as np

SPECIAL = [
    "inf", "-inf", "+inf", "Infinity", "-iNfInItY", "INF", "nan", "-nan", "+NaN", "NAN", "in", "infin", "nana",
    "infinityy", "", " ", ".", "-", "+", "e5", ".e1", "1e", "1e+", "1e-", "1_0", "1__0", "_1", "1_", "1_.5",
    "1._5", "1e_5", "1e5_0", "1e+_5", "0.000_1", "1_0.5_5e+0_1", "00001_0", "1.5.5", "--1", "+-1", "- 1", " 1 ",
    "\t-2.5\x0b", "\x0c3\x0c", "1 2", "1d5", "0x10", "1f", "\x001", "1e99999999999", "-1e-99999999", "0e999999",
    "-0", "+0", "-0.0e-500", "0.0", "000", ".5", "5.", "-.5e1", "1.e5", "1E5", "1e0005",
    "4.9406564584124654e-324", "4.9406564584124654e-325", "2.4703282292062327e-324", "2.4703282292062328e-324",
    "2.470328229206232720882538e-324", "1.7976931348623157e308", "1.7976931348623158e308",
    "1.7976931348623159e308", "1.797693134862315807937289714053e308", "2.2250738585072011e-308",
    "2.2250738585072012e-308", "2.2250738585072014e-308", "9007199254740993", "9007199254740992.5",
    "9007199254740993.0000000000000000000001", "123456789012345678901234567890", "1e22", "1e23", "8.5e-323",
    "0.1", "0.2", "0.3", "1.1", "3.14159", "1e-7", "123.456e-2", "100000000000000000000000000000000",
]


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _from_bits(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def _midpoint_token(rng: random.Random) -> str:
    e = rng.choice([0, 1, 2, rng.randint(1, 2045), 2045, rng.randint(900, 1100)])
    b = (e << 52) | rng.getrandbits(52)
    x, y = Fraction(_from_bits(b)), Fraction(_from_bits(b + 1))
    mid = (x + y) / 2
    getcontext().prec = 800
    s = format(Decimal(mid.numerator) / Decimal(mid.denominator), "e")
    nd = rng.choice([None, 16, 17, 18, 19, 20, 21, 25, 40, 100, 400])
    if nd:
        man, ex = s.split("e")
        digs = man.replace(".", "").replace("-", "")[:nd]
        if rng.random() < 0.35:
            digs = digs[:-1] + str((int(digs[-1]) + rng.choice([1, 9])) % 10)
        s = digs[0] + "." + digs[1:] + "e" + ex
    return ("-" if rng.random() < 0.3 else "") + s


def _digit_token(rng: random.Random) -> str:
    n = rng.randint(1, 60) if rng.random() < 0.9 else rng.randint(700, 900)
    s = "".join(rng.choice("0123456789") for _ in range(n))
    if rng.random() < 0.5:
        p = rng.randint(0, n)
        s = s[:p] + "." + s[p:]
    if rng.random() < 0.6:
        s += rng.choice("eE") + rng.choice(["", "+", "-"]) + str(rng.randint(0, 400))
    if rng.random() < 0.1 and n > 2:
        k = rng.randint(1, len(s) - 1)
        s = s[:k] + "_" + s[k:]
    return rng.choice(["", "-", "+"]) + s


def tokens(seed: int, n: int) -> list[str]:
    """n tokens (no ',', '#', CR or LF in any of them)."""
    rng = random.Random(seed)
    out = list(SPECIAL)
    while len(out) < n:
        k = rng.random()
        if k < 0.3:
            x = _from_bits(rng.getrandbits(63)) if rng.random() < 0.5 else rng.uniform(-10, 10) * 10 ** rng.randint(-30, 30)
            if x != x or abs(x) == float("inf"):
                x = 1.5
            fmt = rng.choice(["%.18e", "%.17g", "%r", "%.25e", "%.40e", "%.3e", "%.0e", "%.60g", "%.20f", "%.16e"])
            out.append(repr(x) if fmt == "%r" else fmt % x)
        elif k < 0.6:
            out.append(_midpoint_token(rng))
        elif k < 0.85:
            out.append(_digit_token(rng))
        else:
            x = _from_bits(rng.getrandbits(52) | (rng.choice([0, 1, 2, 2046, 2045, 1023]) << 52))
            out.append(rng.choice(["%.17g", "%.18e", "%.30e", "%.760e"]) % x)
    return out[:n]


def savetxt_bytes(a: np.ndarray) -> bytes:
    """np.savetxt(fmt='%.18e', delimiter=',') layout, as in the reference's
    example files."""
    rows = ["%s\n" % ",".join("%.18e" % v for v in r) for r in np.atleast_2d(a)]
    return "".join(rows).encode("ascii")


# (text, keyword arguments) covering genfromtxt's line handling
STRUCT_CASES = [
    (b"1,2\n3,4\n", {}),
    (b"1,2\n\n3,4\n", {}),
    (b"1,2 # c\n#x\n3,4", {}),
    (b" 1 , 2 \n3,4", {}),
    (b"1,abc\n3,4", {}),
    (b"1,\n3,4", {}),
    (b"1,2\r\n3,4\r\n", {}),
    (b"1,2\r3,4", {}),
    (b"1,2\r", {}),
    (b"1,2\r\n\r\n3,4\r", {}),
    (b"1,2,3\n3,4", {}),
    (b"inf,-Infinity\nnan,+NaN", {}),
    (b"1,2\n   \n3,4", {}),
    (b"1,2\n\t\n3,4", {}),
    (b"\n\n1,2", {}),
    (b"1,2\n3", {}),
    (b"1\n2\n3", {}),
    (b"5", {}),
    (b"", {}),
    (b"# only\n\n  \n", {}),
    (b"h1,h2\n1,2\n3,4", {"skip_header": 1}),
    (b"1,2\n3,4", {"skip_header": 5}),
    (b"1,2\n3,4,5\n6\n7,8\n", {}),
    (b"\n\n1,2\n\n3\n#c\n4,5,6\n", {}),
    (b"a\nb\n1,2\n3\n", {"skip_header": 2}),
    (b"1;2\n3;4", {"delimiter": ";"}),
    (b"1 2\n3 4", {"delimiter": " "}),
    (b" 1 2 \n3  4\n", {"delimiter": " "}),
    (b"1\t2\n\t3\t4", {"delimiter": "\t"}),
    (b"1,2#3\n4,5#6", {"comments": None}),
    (b"1,2%3\n4,5", {"comments": "%"}),
    (b",\n,", {}),
    (b"1,2\n3,4\n\n\n", {}),
    (b"  # lead\n 7 , 8 ,9\n1e3,  -2_0 ,.5\n", {}),
]


def long_line_case(ncols: int = 5000, seed: int = 0) -> bytes:
    """Two lines whose bytes exceed one CTA's shared-memory stage."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((2, ncols)) * 10.0 ** rng.integers(-300, 300, (2, ncols))
    return savetxt_bytes(a)
