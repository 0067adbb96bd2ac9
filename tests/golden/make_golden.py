"""Writes the golden bound-and-split fixtures of tests/golden/ from the
reference's own code: src/base/Patch.cpp and src/base/Projection.cpp of the
reference tree compiled by oracle/build_ref.sh into oracle/_ref/, driven by
the LIFO loop of src/Reyes/BoundNSplitCLCPU.cpp:75-159 (oracle/ref_pin.cpp).

Each fixture holds the inputs (control points, patch type, modelview,
options) and the reference's emitted sub-patch sequence (patch id and range,
in emission order), so the tests need neither the reference tree nor the
scene generators.  For three of the cases, gpucrit_<case>.npz holds the
sub-patch set of the reference's GPU bound criterion on the same inputs:
bound() of kernels/bound_n_split.h compiled as C++ (oracle/clshim/, driven
by oracle/ref_kernels.cpp).  Run here, where the reference tree exists:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def cases():
    from micropolis_gb300 import scenes
    hf = scenes.heightfield_1024x768()
    mixed = scenes.mixed4096_1920x1080(n=96, width=512, height=512)
    low = scenes.heightfield_1024x768()
    low.width, low.height = 512, 384
    low.draws[0].mv = scenes.look_at((0.0, -0.3, 0.05), (0.0, 1.0, 0.0), (0, 0, 1))
    return [
        ("heightfield_1024x768", hf, 0, {}),
        ("mixed96_bezier_512", mixed, 0, {}),
        ("mixed96_gregory_512", mixed, 1, {}),
        ("mixed96_gregory_depth3_512", mixed, 1, {"max_split_depth": 3}),
        ("heightfield_eye_plane_512x384", low, 0, {"max_split_depth": 12}),
    ]


GPU_CRITERION_CASES = ("mixed96_bezier_512", "mixed96_gregory_512", "heightfield_eye_plane_512x384")


def _one_draw(sc, k):
    from micropolis_gb300 import scenes
    return scenes.Scene(sc.name, sc.width, sc.height, [sc.draws[k]], fovy=sc.fovy, near=sc.near,
                        options=dict(sc.options))


def main():
    from oracle import oracle
    oracle.build_ref()
    if oracle.ref_pin() is None:
        raise SystemExit("the reference tree is needed (oracle/build_ref.sh)")
    for name, sc, k, over in cases():
        p = oracle.make_params(sc, **over)
        pid, rng = oracle.ref_bound_n_split(sc, k, params=p)
        d = sc.draws[k]
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            cp=np.ascontiguousarray(d.mesh.cp, np.float32), type=np.int32(d.mesh.type),
            mv=np.ascontiguousarray(d.mv, np.float32), width=np.int32(sc.width), height=np.int32(sc.height),
            fovy=np.float32(sc.fovy), near=np.float32(sc.near), limit=np.float32(p.bound_n_split_limit),
            cull_ribbon=np.float32(p.cull_ribbon), max_split_depth=np.int32(p.max_split_depth),
            pid=pid.astype(np.int32), range=rng.astype(np.float32))
        print(name, len(pid))
        if name in GPU_CRITERION_CASES:
            q = oracle.make_params(sc, bound_criterion=1, **over)
            gsc = _one_draw(sc, k)
            gpid, grng = oracle.ref_bound_n_split_gpu(gsc, 0, params=q)
            np.savez_compressed(os.path.join(HERE, "gpucrit_" + name + ".npz"), pid=gpid.astype(np.int32),
                                range=grng.astype(np.float32))
            print("gpucrit_" + name, len(gpid))


if __name__ == "__main__":
    main()
