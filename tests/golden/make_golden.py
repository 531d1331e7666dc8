"""Generates the committed golden fixtures from the reference's own data.

Run in a container where the reference tree is mounted (it is read only):
    python tests/golden/make_golden.py [reference_root]
(default: $TDM_REFERENCE_ROOT, else /root/reference)

Writes, next to this script:
  sampledata.npz   P1h, P2h (4x441) and T (4x4) of
                   core/external/estimateRigidTransform/sampleData.mat, the
                   known-answer case of demoEstimateRigidTransform.m.
  sample_clouds.json  for data/sample/3dmatch-demo/single-depth-{1,2}.ply:
                   vertex count, first/last points, bounding box, and the
                   grid geometry core/demo.cu:97-124 derives (dims, origin);
                   plus, per index-decode mode of core/demo.cu:32-34, how many
                   voxels are decoded to a wrong (x,y,z).
Only derived numbers and the small .mat arrays are stored, never the clouds.
"""
import json
import os
import sys

import numpy as np
import scipy.io

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402


def main(ref=os.environ.get("TDM_REFERENCE_ROOT", "/root/reference")):
    d = scipy.io.loadmat(os.path.join(ref, "core/external/estimateRigidTransform/sampleData.mat"))
    np.savez_compressed(os.path.join(HERE, "sampledata.npz"), P1h=d["P1h"], P2h=d["P2h"], T=d["T"])
    clouds = {}
    for f in ("single-depth-1.ply", "single-depth-2.ply"):
        pts = O.read_ply(os.path.join(ref, "data/sample/3dmatch-demo", f))
        dim, origin = O.grid_setup(pts, 0.01, 15)
        clouds[f] = {
            "n": int(pts.shape[0]),
            "first": pts[0].tolist(), "last": pts[-1].tolist(),
            "min": pts.min(0).tolist(), "max": pts.max(0).tolist(),
            "dim": dim.tolist(), "origin": origin.tolist(),
            "misdecoded_float32": O.count_misdecoded(dim, 1),
            "misdecoded_fma": O.count_misdecoded(dim, 2),
        }
    with open(os.path.join(HERE, "sample_clouds.json"), "w") as fh:
        json.dump(clouds, fh, indent=1)


if __name__ == "__main__":
    main(*(sys.argv[1:2]))
