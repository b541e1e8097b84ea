"""Fixtures from the reference's own scene-regression files
(data/regression/*.json[.gz], compared by projects/regressionTests/
regressionTests.cpp:45-102) and the meshes they name.

    python tests/golden/make_regression.py

Writes, per scene, regression_<scene>.npz with the rest mesh, the recorded
frame numbers and the recorded displacement and velocity of every `stride`-th
frame (plus the first three and the last), and <scene>_head.json.gz: the
file's scene object and first three frames unchanged, for the JSON reader.
Reads the reference checkout at /root/reference (this container only)."""
import gzip
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from hobakv1_gb300.replay import read_tobj  # noqa: E402

REF = "/root/reference"
SCENES = {"newmark_stretch": ("data/regression/newmark_stretch.json.gz", "data/cube_10.tobj", 3)}


def main():
    for name, (rec, mesh, stride) in SCENES.items():
        with gzip.open(os.path.join(REF, rec), "rt") as f:
            doc = json.load(f)
        rest, tets = read_tobj(os.path.join(REF, mesh))
        frames = doc["frames"]
        n = len(frames)
        keep = sorted(set([0, 1, 2, n - 1] + list(range(0, n, stride))))
        np.savez_compressed(
            os.path.join(HERE, f"regression_{name}.npz"), rest=rest, tets=tets, dt=doc["scene"]["dt"],
            total_frames=n, frames=np.array(keep),
            frame_number=np.array([frames[k]["frameNumber"] for k in keep]),
            position=np.array([frames[k]["position"] for k in keep]),
            velocity=np.array([frames[k]["velocity"] for k in keep]))
        with gzip.open(os.path.join(HERE, f"{name}_head.json.gz"), "wt") as f:
            json.dump({"scene": doc["scene"], "frames": frames[:3]}, f)
        print(name, n, "frames,", len(keep), "kept")


if __name__ == "__main__":
    main()
