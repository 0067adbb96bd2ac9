#!/bin/sh
# Compiles the reference's own src/base/Patch.cpp and src/base/Projection.cpp
# from the reference tree (read in place, never copied) together with the pin
# driver ref_pin.cpp, and the reference's kernels (rewritten for C++ into
# oracle/_ref/kernels/, outside the repository's history) with the CPU
# work-item runtime ref_kernels.cpp, into oracle/_ref/libref_pin.so.  The reference's other
# sources need OpenCL, OpenGL, GLFW, boost, capnp and generated config headers
# and are not compiled.  The tree is named by MP_REFERENCE_DIR; the script
# skips quietly when that variable is unset or names no reference tree.
#
# The CPU sources compile without floating-point contraction (the reference's
# CPU build on x86 has none).  The kernels compile with contraction on, as
# OpenCL C compiles them (FP_CONTRACT defaults to ON); x86 needs -mfma for
# gcc to emit fused multiply-adds, Arm has them in its base instruction set.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${MP_REFERENCE_DIR:-}
[ -n "$REF" ] || { echo "build_ref: MP_REFERENCE_DIR is not set, skipped"; exit 0; }
[ -f "$REF/src/base/Patch.cpp" ] || { echo "build_ref: no reference tree at $REF, skipped"; exit 0; }
OUT="$HERE/_ref"
mkdir -p "$OUT/obj"
FMA=
case $(uname -m) in x86_64|amd64) FMA=-mfma ;; esac
COMMON="-std=c++17 -O2 -fno-fast-math -fwrapv -fPIC -w -pthread"
PIDS=
for f in "$REF/src/base/Patch.cpp" "$REF/src/base/Projection.cpp" "$HERE/ref_pin.cpp"; do
    g++ $COMMON -ffp-contract=off -I "$HERE/refshim" -I "$REF/src/base" -I "$HERE" -c "$f" \
        -o "$OUT/obj/$(basename "$f" .cpp).o" &
    PIDS="$PIDS $!"
done
# The reference's kernels (kernels/*.cl) rewritten into C++ by clshim/rewrite.py,
# into _ref/kernels/ only, then compiled with the fiber runtime ref_kernels.cpp.
python3 "$HERE/clshim/rewrite.py" "$REF/kernels" "$OUT/kernels"
# the oracle's sine stands for native_sin (clshim/cl_shim.h)
g++ $COMMON -ffp-contract=off -fopenmp -c "$HERE/oracle.cpp" -o "$OUT/obj/oracle.o" &
PIDS="$PIDS $!"
g++ $COMMON $FMA -ffp-contract=fast -I "$HERE" -c "$HERE/ref_kernels.cpp" -o "$OUT/obj/ref_kernels.o"
for p in $PIDS; do wait "$p"; done
g++ -shared -pthread -fopenmp "$OUT/obj/Patch.o" "$OUT/obj/Projection.o" "$OUT/obj/ref_pin.o" \
    "$OUT/obj/ref_kernels.o" "$OUT/obj/oracle.o" -o "$OUT/libref_pin.so"
# where the pin came from, for the tests that read the reference's own files
# (its test scenes, its trace tools) and skip where the tree is absent
printf '%s\n' "$REF" > "$OUT/reference_dir.txt"
echo "build_ref: $OUT/libref_pin.so"
