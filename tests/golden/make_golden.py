"""Generate the golden fixtures in this directory (run from the repository root):

    python tests/golden/make_golden.py

golden_map_coordinates.npz -- scipy.ndimage.map_coordinates(order=1, mode="nearest")
outputs on seeded 1-D and 2-D grids, including coordinates outside [0, G-1] on both
sides and exact grid nodes. The reference evaluates its VM tensors through
jax.scipy.ndimage.map_coordinates with exactly these arguments (tensorf/tensor_vm.py:
242-248); jax documents that function as matching scipy's for order <= 1. These
fixtures pin the oracle's interpolation to an implementation independent of it.
"""
import os

import numpy as np
from scipy import ndimage

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    rng = np.random.default_rng(20240601)
    out = {}
    for g in (2, 5, 17):
        line = rng.normal(size=(g,))
        plane = rng.normal(size=(g, g))
        c1 = np.concatenate([rng.uniform(-1.5, g + 0.5, size=40), np.arange(g, dtype=np.float64),
                             [-0.7, -1e-7, g - 1 + 1e-7, g - 1.0, g + 3.2]])
        c2 = np.stack([rng.uniform(-1.5, g + 0.5, size=60), rng.uniform(-1.5, g + 0.5, size=60)])
        c2 = np.concatenate([c2, np.array([[-0.7, 4.6 if g > 4 else 1.2, 0.0, g - 1.0],
                                           [g - 1.0, -0.3, 0.0, g + 0.7]])], axis=1)
        out[f"line_{g}"] = line
        out[f"plane_{g}"] = plane
        out[f"c1_{g}"] = c1
        out[f"c2_{g}"] = c2
        out[f"y1_{g}"] = ndimage.map_coordinates(line, c1[None], order=1, mode="nearest")
        out[f"y2_{g}"] = ndimage.map_coordinates(plane, c2, order=1, mode="nearest")
    np.savez(os.path.join(HERE, "golden_map_coordinates.npz"), **out)


if __name__ == "__main__":
    main()
