"""Generate the oracle golden fixtures of tests/test_golden.py.

The reference has no golden vectors of its own (no tests, no fixtures), so
these pin the oracle itself: outputs of the CPU oracle on seeded synthetic
scenes, frozen so that any change of the restated maths, and any difference
between x86-64 and aarch64 builds of the oracle, is caught.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from voxel_cone_tracing_gb300 import scenes  # noqa: E402

CASES = {
    # name: (scene builder, params)
    "small_ref_aniso": (lambda: scenes.scene_small(seed=1000, width=48, height=32),
                        dict(grid_res=32, width=48, height=32, vox_mode=O.VOX_REF_RASTER2X, mip_mode=O.MIP_ANISO)),
    "small_sat_iso_six": (lambda: scenes.scene_small(seed=1001, width=48, height=32),
                          dict(grid_res=32, width=48, height=32, vox_mode=O.VOX_CONSERVATIVE, mip_mode=O.MIP_ISO,
                               cone_set=O.CONES_SIX60)),
    "sphere_ref_aniso": (lambda: scenes.scene_sphere(seed=2000, freq=12, width=40, height=24),
                         dict(grid_res=32, width=40, height=24)),
}


def compute(name):
    build, kw = CASES[name]
    scene = build()
    p = O.Params(threads=4, **kw)
    r = O.render(scene, p)
    return dict(level0=r["level0"], counts=r["counts"], chains=r["chains"], tri_id=r["gbuffer"]["tri_id"],
                frame=r["frame"])


def main():
    for name in CASES:
        out = compute(name)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
