"""Writes rsc_sincos_table.h: sin(j / 64) and cos(j / 64), j = 0 .. 52, each
as a double-float (head = the value rounded to FP32, tail = the remainder
rounded to FP32), computed with mpmath at 60 digits.  The compensated pulse
evaluates the sine and cosine of its reduced phase r as those of the nearest
node j / 64 combined with short series in d = r - j / 64 (|d| <= 1/128).

Run from this folder:  python gen_sincos_table.py > rsc_sincos_table.h
"""
import struct

import mpmath

mpmath.mp.dps = 60
NODES = 53          # |r| <= pi / 4 + a little: j up to 51; one spare
STEP = 64


def f32(x):
    return struct.unpack("<f", struct.pack("<f", float(x)))[0]


def split(v):
    hi = f32(v)
    lo = f32(v - mpmath.mpf(hi))
    return hi, lo


def hexf(x):
    """A C hex-float literal of an FP32 value (mantissa without trailing zeros)."""
    if x == 0.0:
        return "0.0f"
    m, e = float(x).hex().split("p")
    m = m.rstrip("0").rstrip(".")
    return "%sp%sf" % (m, e)


def main():
    print("/* rsc_sincos_table.h -- written by gen_sincos_table.py (mpmath, 60 digits).")
    print(" * kSinCosNode[j] = {sin hi, sin lo, cos hi, cos lo} of j / %d. */" % STEP)
    print("#ifndef SIMRADAR_GB300_RSC_SINCOS_TABLE_H")
    print("#define SIMRADAR_GB300_RSC_SINCOS_TABLE_H")
    print("constexpr int kSinCosNodes = %d;" % NODES)
    print("constexpr float kSinCosStep = %d.0f;" % STEP)
    print("__device__ const float4 kSinCosNode[kSinCosNodes] = {")
    for j in range(NODES):
        t = mpmath.mpf(j) / STEP
        sh, sl = split(mpmath.sin(t))
        ch, cl = split(mpmath.cos(t))
        print("    {%s, %s, %s, %s}," % (hexf(sh), hexf(sl), hexf(ch), hexf(cl)))
    print("};")
    print("#endif")


if __name__ == "__main__":
    main()
