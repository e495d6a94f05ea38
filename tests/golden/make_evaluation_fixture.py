"""Extracts a small fixture from the reference's own simulation outputs of its dihedral
evaluation (evaluation/simulation/dihedral-{5,7,10,15}cm: 601 poses x 256 range bins of
complex64, chirp 0 / channel 0 of a guided PathTracer run of the examples/src/1_dihedral.cpp
setup over azimuths linspace(-75, 75, 601), as evaluation/OurMeasurements.ipynb reads
them). Kept: every 4th pose (151 of 601) and range bins 8..31 (the reflector's return
sits at bin 20), as complex64 -> tests/golden/dihedral_eval_ref.npz.

Usage: HUSSAR_REFERENCE=<reference checkout> python tests/golden/make_evaluation_fixture.py
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SIZES_MM = (50, 70, 100, 150)
POSE_STEP = 4
BINS = (8, 32)


def main():
    ref = os.environ["HUSSAR_REFERENCE"]
    out = {}
    for s in SIZES_MM:
        d = np.fromfile(os.path.join(ref, "evaluation", "simulation", "dihedral-%dcm" % (s // 10)),
                        np.complex64).reshape(-1, 256)
        assert d.shape == (601, 256)
        out["size%d" % s] = np.ascontiguousarray(d[::POSE_STEP, BINS[0]:BINS[1]])
    angles = np.linspace(-75.0, 75.0, 601)[::POSE_STEP]
    np.savez_compressed(os.path.join(HERE, "dihedral_eval_ref.npz"), angles_deg=angles,
                        bins=np.arange(*BINS), sizes_mm=np.array(SIZES_MM), **out)
    print("wrote", os.path.join(HERE, "dihedral_eval_ref.npz"))


if __name__ == "__main__":
    main()
