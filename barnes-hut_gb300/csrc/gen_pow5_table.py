#!/usr/bin/env python3
"""Writes bh_pow5_table.h: 128-bit approximations of 5^q, q = -342 .. 308,
for the decimal-to-binary64 conversion of the GPU CSV reader.

Entry q holds F (hi, lo 64-bit halves, 2^127 <= F < 2^128) and s with
    q >= 0:  F = floor(5^q / 2^s)            (exact for q <= 55, s <= 0)
    q <  0:  F = ceil(2^-s / 5^-q)           (s = -(127 + bitlen(5^-q)))
so that F * 2^s approximates 5^q from below (q >= 0) or above (q < 0) to
within one unit of F's last bit.

    python barnes-hut_gb300/csrc/gen_pow5_table.py > barnes-hut_gb300/csrc/bh_pow5_table.h
"""
QMIN, QMAX = -342, 308


def entry(q):
    if q >= 0:
        p = 5 ** q
        b = p.bit_length()
        return (p << (128 - b), b - 128) if b <= 128 else (p >> (b - 128), b - 128)
    d = 5 ** (-q)
    t = 127 + d.bit_length()
    return -((-(1 << t)) // d), -t


def main():
    hi, lo, sh = [], [], []
    for q in range(QMIN, QMAX + 1):
        f, s = entry(q)
        assert (1 << 127) <= f < (1 << 128)
        hi.append(f >> 64)
        lo.append(f & ((1 << 64) - 1))
        sh.append(s)
    out = ["// Generated by gen_pow5_table.py (same folder); do not edit.",
           "// 128-bit approximations F * 2^s of 5^q, q = -342 .. 308: see the generator.",
           "#pragma once", "", "#include <cstdint>", "",
           f"constexpr int kPow5Min = {QMIN};", f"constexpr int kPow5Max = {QMAX};",
           "constexpr int kPow5ExactMax = 55;  // F * 2^s == 5^q exactly for 0 <= q <= 55", ""]

    def arr(name, typ, vals, fmt, per):
        out.append(f"__device__ const {typ} {name}[{len(vals)}] = {{")
        for i in range(0, len(vals), per):
            out.append("    " + ", ".join(fmt(v) for v in vals[i:i + per]) + ",")
        out.append("};")
        out.append("")
    arr("kPow5Hi", "uint64_t", hi, lambda v: f"0x{v:016x}ull", 4)
    arr("kPow5Lo", "uint64_t", lo, lambda v: f"0x{v:016x}ull", 4)
    arr("kPow5Shift", "int16_t", sh, str, 12)
    print("\n".join(out))


if __name__ == "__main__":
    main()
