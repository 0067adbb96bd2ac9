#!/bin/sh
# Compiles the reference's own src/base/Patch.cpp and src/base/Projection.cpp
# from the reference tree (read in place, never copied) together with the pin
# driver ref_pin.cpp into oracle/_ref/libref_pin.so.  The reference's other
# sources need OpenCL, OpenGL, GLFW, boost, capnp and generated config headers
# and are not compiled.  Skips quietly when the reference tree is absent.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${MP_REFERENCE_DIR:-/root/reference}
[ -f "$REF/src/base/Patch.cpp" ] || { echo "build_ref: no reference tree at $REF, skipped"; exit 0; }
mkdir -p "$HERE/_ref"
g++ -std=c++14 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -w \
    -I "$HERE/refshim" -I "$REF/src/base" \
    "$REF/src/base/Patch.cpp" "$REF/src/base/Projection.cpp" "$HERE/ref_pin.cpp" \
    -o "$HERE/_ref/libref_pin.so"
echo "build_ref: $HERE/_ref/libref_pin.so"
