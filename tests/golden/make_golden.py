"""Regenerates tests/golden/example01_map_slices.npz from the reference's own
recorded boundary-map images (CUDASPHNEW/distances.ppm, viscosities.ppm:
mid-z slices of Example01's box maps written by
SphInComplexShapes::SaveSliced{Distance,Viscosity}MapToPpm via
particle_simulation.cu:2613-2614).  Run once where the reference checkout is
available, with the path of its CUDASPHNEW directory:

    python tests/golden/make_golden.py <reference checkout>/CUDASPHNEW
"""
import os
import sys

import numpy as np


def load_ppm(path):
    toks = open(path).read().split()
    assert toks[0] == "P3"
    w, h, _ = int(toks[1]), int(toks[2]), int(toks[3])
    return np.array(toks[4:4 + 3 * w * h], dtype=np.int64).reshape(h, w, 3).astype(np.uint8)


def main(ref_dir):
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "example01_map_slices.npz")
    np.savez_compressed(out,
                        distances=load_ppm(os.path.join(ref_dir, "distances.ppm")),
                        viscosities=load_ppm(os.path.join(ref_dir, "viscosities.ppm")))
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1])
