"""Rewrites OpenCL C source on stdin into the C++ that opencl_c.hpp compiles,
line for line, on stdout (test infrastructure; used by oracle/ref/Makefile to
compile the reference's rs.cl where it lies, nothing is written to disk).

Two spellings of OpenCL C have no C++ reading and are rewritten:
  - swizzles:       v.xyz  v.s012  v.hi  v.sb   ->  v.xyz()  v.s012()  v.hi()  v.sb()
  - vector literals and casts:
                    (float4)(a, b, c)            ->  float4_make(a, b, c)
                    (float4)r   (float4)d.s0     ->  float4_make(r)  float4_make(d.s0())
Everything else, comments included, is passed through unchanged.
"""
import re
import sys

VEC = r"(?:float|u?int|u?char|u?short|u?long|double)(?:2|3|4|8|16)"
SWIZZLE = re.compile(r"\.(s[0-9a-fA-F]+|[xyzw]{1,4}|lo|hi|even|odd)\b(?!\s*\()")
LITERAL = re.compile(r"\(\s*(" + VEC + r")\s*\)\s*\(")
CAST = re.compile(r"\(\s*(" + VEC + r")\s*\)\s*([A-Za-z_]\w*(?:\[[^\]]*\])?(?:\.\w+\(\))*)")


def convert(line):
    line = SWIZZLE.sub(r".\1()", line)
    line = LITERAL.sub(r"\1_make(", line)
    return CAST.sub(r"\1_make(\2)", line)


def main():
    for line in sys.stdin:
        sys.stdout.write(convert(line))


if __name__ == "__main__":
    main()
