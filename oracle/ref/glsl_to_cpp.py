"""Turns one of the reference's GLSL shaders into a C++ translation unit for glsl_shim.h (test
infrastructure: run by oracle/Makefile, output only under oracle/_ref/).

The shader text is kept as written except for five mechanical changes: the GLSL-only lines
(#version, #extension, precision) are dropped, decimal literals get an `f` suffix (GLSL literals are
single precision, C++ ones double), a multi-component swizzle that is read (not assigned to) gets
glm's call syntax `v.xyz()` (glm's swizzle proxies do not convert implicitly inside its templated
functions and operators), the stage's `in` / `out` variables become thread_local globals (one
invocation per host thread at a time), and the shim header is included first.

usage: python glsl_to_cpp.py SHADER OUT.cpp
"""
import re
import sys

STAGE_VARIABLE = re.compile(r"^\s*(?:layout\s*\([^)]*\)\s*)?(?:in|out)\s+(\w+\s+\w+\s*;.*)$")
SWIZZLE_READ = re.compile(r"\.([xyzw]{2,4}|[rgba]{2,4})\b(?!\s*(?:\(|[-+*/]?=(?!=)))")
FLOAT_LITERAL = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][-+]?\d+)?|\d+[eE][-+]?\d+|\.\d+(?:[eE][-+]?\d+)?)(?![\w.])")


def convert(text):
    out = ['#include "glsl_shim.h"']
    for line in text.splitlines():
        s = line.strip()
        if s.startswith("#version") or s.startswith("#extension") or s.startswith("precision "):
            out.append("// (GLSL only) " + s)
            continue
        if s.startswith("//"):
            out.append(line)
            continue
        m = STAGE_VARIABLE.match(line)
        if m:
            line = "thread_local " + m.group(1)
        code, sep, comment = line.partition("//")
        code = FLOAT_LITERAL.sub(lambda m: m.group(1) + "f", code)
        code = SWIZZLE_READ.sub(lambda m: "." + m.group(1) + "()", code)
        out.append(code + sep + comment)
    return "\n".join(out) + "\n"


def main():
    src, dst = sys.argv[1], sys.argv[2]
    with open(src) as f:
        text = f.read()
    with open(dst, "w") as f:
        f.write(convert(text))


if __name__ == "__main__":
    main()
