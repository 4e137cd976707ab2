"""Generate csv_pow10.cuh: 128-bit truncations of the powers of ten used by
the CSV reader's decimal-to-binary conversion (csv.cu).

For every q in [-342, 308]:  10^q = (T + eps) * 2^b  with  T an integer in
[2^127, 2^128), 0 <= eps < 1, and eps == 0 exactly when 0 <= q <= 55
(5^q < 2^128).  Python integers make every entry exact; run

    python arbinterp_gb300/csrc/gen_pow10.py

to rewrite the header (the build does so when it is missing).
"""
import os

QMIN, QMAX = -342, 308


def entry(q):
    if q >= 0:
        v = 10 ** q
        bl = v.bit_length()
        if bl <= 128:
            return v << (128 - bl), bl - 128
        return v >> (bl - 128), bl - 128
    d = 10 ** (-q)
    s = 127 + d.bit_length()
    return (1 << s) // d, -s


def main(path=None):
    path = path or os.path.join(os.path.dirname(os.path.abspath(__file__)), "csv_pow10.cuh")
    rows, exps = [], []
    for q in range(QMIN, QMAX + 1):
        t, b = entry(q)
        assert (1 << 127) <= t < (1 << 128) - 1, q
        # the identity the table encodes, checked exactly
        if q >= 0:
            exact = 10 ** q == t * 2 ** b if b >= 0 else 10 ** q * 2 ** (-b) == t
            assert (b >= 0 and t * 2 ** b <= 10 ** q < (t + 1) * 2 ** b) or (b < 0 and exact), q
            assert exact == (q <= 55), q
        else:
            assert t * 10 ** (-q) <= 2 ** (-b) < (t + 1) * 10 ** (-q), q
        rows.append("  {0x%016xULL, 0x%016xULL}," % (t >> 64, t & ((1 << 64) - 1)))
        exps.append(str(b))
    out = [
        "// Generated by gen_pow10.py: 10^q = (T + eps) * 2^b, T in [2^127, 2^128),",
        "// 0 <= eps < 1 (eps == 0 for 0 <= q <= 55).  Do not edit.",
        "#pragma once",
        "#include <stdint.h>",
        "namespace arb {",
        "namespace csv {",
        "constexpr int kPow10Min = %d, kPow10Max = %d;" % (QMIN, QMAX),
        "__device__ const uint64_t kPow10T[%d][2] = {" % (QMAX - QMIN + 1),
        *rows,
        "};",
        "__device__ const int16_t kPow10B[%d] = {" % (QMAX - QMIN + 1),
    ]
    for i in range(0, len(exps), 16):
        out.append("  " + ", ".join(exps[i:i + 16]) + ",")
    out += ["};", "}  // namespace csv", "}  // namespace arb", ""]
    with open(path, "w") as f:
        f.write("\n".join(out))
    return path


if __name__ == "__main__":
    print(main())
