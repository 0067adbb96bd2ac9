"""Rewrites the reference's OpenCL C kernels (kernels/utility.h, dice.cl,
reyes.cl, framebuffer.cl, bound_n_split.h) into C++ that compiles over cl_shim.h, into
oracle/_ref/kernels/ (never into the repository): TEST INFRASTRUCTURE ONLY.

Only what C++ cannot express through the shim is rewritten:
  * vector literals (float4)(a, b, c, d) become constructor calls float4(...);
  * work-group local variables (`local T x;` in a kernel body) become
    `static thread_local` (one work-group runs on one host thread at a time);
  * `volatile global` buffers lose the volatile (their atomics go through the
    shim, plain stores need no volatile);
  * OpenCL's component-wise ?: on an int3 condition becomes vselect3();
  * the scalar float divisions (p.x/p.w, depth / 200.0f and the four of
    outside_frustum) become cl_fdiv() and the (int) casts of floats cl_f2i(),
    the shim's fixed choices for what -cl-fast-relaxed-math leaves open.
Everything else (swizzles, built-ins, operators) is the shim's.

    python oracle/clshim/rewrite.py <reference kernels dir> <output dir>
"""
import os
import re
import sys

FILES = ("utility.h", "dice.cl", "reyes.cl", "framebuffer.cl", "bound_n_split.h")


def rewrite(text: str) -> str:
    text = re.sub(r"\((float|int)(2|3|4|16)\)\s*\(", r"\1\2(", text)
    text = re.sub(r"^(\s*)(volatile\s+)?local\s+", lambda m: m.group(1) + "static thread_local " + (m.group(2) or ""),
                  text, flags=re.M)
    text = re.sub(r"volatile\s+(__)?global\b", "global", text)
    text = re.sub(r"(\([^;?]*\))\s*\?\s*int3\(\s*-1\s*,\s*-1\s*,\s*-1\s*\)\s*:\s*int3\(\s*0\s*,\s*0\s*,\s*0\s*\)",
                  r"vselect3(\1, int3(-1, -1, -1), int3(0, 0, 0))", text)
    text = re.sub(r"\b(p\.[xyz])/p\.w\b", r"cl_fdiv(\1, p.w)", text)
    text = re.sub(r"\bdepth / 200\.0f", "cl_fdiv(depth, 200.0f)", text)
    text = re.sub(r"\b(p(?:min|max)\.[xy])/(\(\(p(?:min|max)\.[xy] [<>] 0\) \? n : f\))", r"cl_fdiv(\1, \2)", text)
    text = re.sub(r"\(int\)\(", "cl_f2i(", text)
    return text


def main(src: str, dst: str) -> None:
    os.makedirs(dst, exist_ok=True)
    for f in FILES:
        with open(os.path.join(src, f)) as fh:
            text = rewrite(fh.read())
        out = f.replace(".cl", ".inc")
        with open(os.path.join(dst, out), "w") as fh:
            fh.write(text)


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
