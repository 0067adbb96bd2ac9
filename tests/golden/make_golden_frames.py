"""Writes golden framebuffers of tests/golden/ from the reference's own
kernels: kernels/dice.cl, kernels/reyes.cl and kernels/framebuffer.cl
compiled as C++ by oracle/build_ref.sh (oracle/clshim/, run by
oracle/ref_kernels.cpp with the launch geometry of src/Reyes/RendererCL.cpp)
after the reference's CPU bound-and-split, on the scenes of the golden
bound-and-split fixtures.

Each frame fixture holds the covered pixels only (tiled framebuffer index,
RGBA colour, integer depth key), the options it was rendered with and the
cleared pixel's colour, which every other pixel holds.  Run here, where the
reference tree exists:

    python tests/golden/make_golden_frames.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

# (fixture case, displacement, reyes_patch_size)
FRAMES = [("mixed96_bezier_512", 0, 8), ("mixed96_bezier_512", 1, 8), ("mixed96_gregory_512", 0, 8),
          ("mixed96_gregory_depth3_512", 1, 8), ("mixed96_bezier_512", 0, 16)]


def frame_name(case, disp, ps):
    return f"frame_{case}_d{disp}_ps{ps}"


def main():
    from oracle import oracle
    from helpers import golden_case
    oracle.build_ref()
    if oracle.ref_pin() is None or not hasattr(oracle.ref_pin(), "refk_render"):
        raise SystemExit("the reference tree is needed (oracle/build_ref.sh)")
    for case, disp, ps in FRAMES:
        sc, _, _, _ = golden_case(case)
        p = oracle.make_params(sc, displacement=disp, reyes_patch_size=ps)
        color, depth, n = oracle.ref_render(sc, params=p)
        idx = np.flatnonzero(depth != 0x7fffffff).astype(np.int32)
        empty = np.flatnonzero(depth == 0x7fffffff)
        assert len(empty) and np.all(color[empty] == color[empty[0]])
        np.savez_compressed(os.path.join(HERE, frame_name(case, disp, ps) + ".npz"),
                            case=np.array(case), displacement=np.int32(disp), patch_size=np.int32(ps),
                            subpatches=np.int64(n), index=idx, color=color[idx].astype(np.float32),
                            depth=depth[idx].astype(np.int32), pixels=np.int64(depth.size),
                            clear=color[empty[0]].astype(np.float32))
        print(frame_name(case, disp, ps), n, len(idx))


if __name__ == "__main__":
    main()
