"""Generate the golden fixtures from the reference engine itself.

Runs the reference (oracle/_ref/libcpref.so, built from the reference's own
sources) on seeded scenes and stores the resulting states and contacts.
Usage: python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from constraintphysics_gb300 import scenes  # noqa: E402


def main():
    steps = 120
    w = oracle.ref_world()
    scenes.apply(scenes.hull_drop(seed=1, n_side=3), w)
    w.step(steps)
    st = w.state()
    c = w.contacts()
    np.savez_compressed(os.path.join(HERE, "hull_drop_3_seed1.npz"), steps=steps, com=st["com"], quat=st["quat"],
                        vel=st["vel"], ang_vel=st["ang_vel"], magic_b=c["magic_b"], b1=c["b1"], b2=c["b2"],
                        normal_impulse=c["normal_impulse"], pen_depth=c["pen_depth"])


if __name__ == "__main__":
    main()
