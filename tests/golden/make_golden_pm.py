"""Writes the photon-mapper fixtures under tests/golden/ from the reference's
own photon mapper (core/src/PhotonMapping.cpp, driven by
oracle/ref_pm_harness.cpp in the build under oracle/_ref; needs the reference
sources, so this runs on the development machine only).

  HASTY_REFERENCE_DIR=<reference checkout> python -m hastyrenderer_gb300.build --oracle
  python tests/golden/make_golden_pm.py

Fixtures: pm_<name>.npz for the golden scenes cornell (area light, glossy
metal), room (area light, glass, texture maps) and field (sky only, no
photons): per progressive iteration 0..3 the colour estimate, normal and
albedo images (H, W, 3), the per-pixel radii (H, W), and the photons emitted
and stored, with the project's keyed random streams (oracle/port/hor_rng.hpp).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import PhotonMapper  # noqa: E402

ITERATIONS = 4
SCENES = ("cornell", "room", "field")


def main():
    for name in SCENES:
        pm = PhotonMapper(os.path.join(HERE, "scenes", name, "renderJob.json"), reference=True)
        out = {k: [] for k in ("color", "normal", "albedo", "radii", "emitted", "stored")}
        for _ in range(ITERATIONS):
            r = pm.iterate(1)
            for k in out:
                out[k].append(r[k])
        pm.close()
        np.savez_compressed(os.path.join(HERE, f"pm_{name}.npz"), **{k: np.array(v) for k, v in out.items()})
    print("photon-mapper fixtures written to", HERE)


if __name__ == "__main__":
    main()
