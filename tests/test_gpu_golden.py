"""GPU: the CUDA solver against the committed golden fixtures (tests/golden/*.npz, made
by the pure-Python restatement), bit for bit — no oracle needed on the GPU machine."""
from pathlib import Path

import numpy as np
import pytest

import velvet_gb300 as vg
from velvet_gb300 import workloads as W
import test_pyref_vs_oracle as scenes

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", sorted(scenes.SCENES))
def test_gpu_matches_golden_fixture(name):
    g = np.load(GOLDEN / f"{name}.npz")
    specs, cfg = scenes.scene_specs(name), scenes.SCENES[name]
    s = vg.ClothSolver(scenes.params_for(name))
    scenes.register(s, specs)
    d = specs[-1].particle_diameter()
    for f in range(cfg["frames"]):
        s.simulate(float(W.FRAME_DT), cfg["substeps"], cfg["iterations"], 1.0, 0.1, 0.06, d)
        s.sync()
        x = s.positions()
        assert np.array_equal(x.view(np.uint32), g["positions"][f].view(np.uint32)), f"{name} frame {f}"
        assert np.array_equal(s.velocities().view(np.uint32), g["velocities"][f].view(np.uint32))
    assert np.array_equal(s.normals().view(np.uint32), g["normals"].view(np.uint32))
