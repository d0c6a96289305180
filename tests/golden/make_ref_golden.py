"""Writes tests/golden/ref_<scene>.npz from the reference's own solver kernels
(Velvet/VtClothSolverGPU.cu and Velvet/SpatialHashGPU.cu compiled unmodified for the CPU,
oracle/_ref/libvr_ref.so, see oracle/refemu/vr_driver.cpp): per scene of tests/ref_scenes.py
the positions and velocities at the recorded frames, the final normals and the last
hash (keys, sorted indices, cell starts); and HashObjects on tests/ref_scenes.HASH_CLOUD.
Needs the reference tree (make -C oracle ref builds the library from it).

    python tests/golden/make_ref_golden.py
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE.parent.parent), str(HERE.parent)]

import ref_scenes  # noqa: E402
import refemu  # noqa: E402


def main():
    if not refemu.available():
        sys.exit("the reference tree is not here: oracle/_ref/libvr_ref.so cannot be built")
    for name in sorted(ref_scenes.SCENES):
        s = refemu.RefSolver(ref_scenes.params_for(name))
        rec, normals = ref_scenes.run(name, s)
        arrays = {"normals": normals}
        for f, (x, v) in rec.items():
            arrays[f"positions_{f}"] = x
            arrays[f"velocities_{f}"] = v
        hv = s.hash_view()
        for k in ("particle_hash", "particle_index", "cell_start"):
            arrays[k] = hv[k]
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        print(name, sorted(rec))
    c = ref_scenes.HASH_CLOUD
    pos, orig = ref_scenes.hash_cloud_inputs()
    h = refemu.hash_objects(pos, orig, c["spacing"], c["table"], c["max_neighbors"], c["diameter"])
    np.savez_compressed(HERE / "ref_hash_cloud.npz", **h)
    print("ref_hash_cloud", h["neighbors"].shape)


if __name__ == "__main__":
    main()
