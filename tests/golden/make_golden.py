"""Writes the golden fixtures tests/golden/<scene>.npz from the pure-Python restatement
(tests/pyref.py) of the reference solver: per scene, the positions and velocities after
every frame and the final normals.  Scenes are defined in tests/test_pyref_vs_oracle.py.

    python tests/golden/make_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE.parent.parent), str(HERE.parent)]

import test_pyref_vs_oracle as scenes  # noqa: E402


def main():
    for name in sorted(scenes.SCENES):
        x, v, n = scenes.run_pyref(name)
        np.savez_compressed(HERE / f"{name}.npz", positions=x, velocities=v, normals=n)
        print(name, x.shape)


if __name__ == "__main__":
    main()
