"""Loads the golden fixtures (tests/golden/*.npz)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: (z[k].item() if z[k].shape == () else z[k]) for k in z.files}
