"""CPU: the C oracle against the independent Python restatement (tests/pyref.py) on tiny
scenes, bit for bit, and both against the committed golden fixtures in tests/golden/
(made by tests/golden/make_golden.py from pyref)."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import oracle
import pyref
from oracle import Oracle
from velvet_gb300 import _abi
from velvet_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"

# name -> (cloth specs, frame settings, parameter overrides)
SCENES = {
    # a flat 5x5 cloth pinned at two corners, draped on a sphere, ground plane
    "drape5": dict(substeps=2, iterations=3, frames=4, params={}),
    # a tilted 6x6 cloth pinned at one corner, bending compliance, hash every 2nd substep
    "fold6": dict(substeps=3, iterations=2, frames=5, params={"interleaved_hash": 2, "bend_compliance": 0.2}),
    # a 4x4 sheet dropped 0.1 m onto another 4x4 sheet lying on the ground: the two
    # cloths of one solver collide (self-collision across cloths, friction)
    "stack2": dict(substeps=2, iterations=2, frames=14, params={}),
}


def scene_specs(name):
    if name == "drape5":
        return [W.ClothSpec(5, 0.05, W.horizontal_cloth(5, 0.05, 0.35), [0, 4],
                            W.static_colliders([W.sphere((0.0, 0.2, 0.0), 0.12), W.plane(0.0)]))]
    if name == "fold6":
        m = W.model_matrix((0.0, 0.2, 0.1), (60.0, 0.0, 0.0))
        return [W.ClothSpec(6, 0.04, m, [0], W.static_colliders([W.plane(0.0)]))]
    if name == "stack2":
        ground = W.static_colliders([W.plane(0.0)])
        return [W.ClothSpec(4, 0.05, W.horizontal_cloth(4, 0.05, 0.07), [], ground),
                W.ClothSpec(4, 0.05, W.model_matrix((0.02, 0.17, 0.085), (90.0, 0.0, 0.0)), [], ground)]
    raise KeyError(name)


def params_for(name):
    p = _abi.VtParams()
    oracle.lib().vo_params_default(C.byref(p))
    for k, v in SCENES[name]["params"].items():
        setattr(p, k, v)
    return p


def register(solver, specs):
    """AddCloth + the cloth object's constraint generation, cloth after cloth."""
    for spec in specs:
        verts, idx = spec.mesh()
        off = solver.add_cloth(verts, idx, spec.model, spec.particle_diameter())
        solver.build_grid_constraints(off, spec.resolution, spec.attached)
    solver.update_colliders(specs[0].colliders(0))


def run_pyref(name):
    specs, cfg = scene_specs(name), SCENES[name]
    cloths = []
    for s in specs:
        verts, idx = s.mesh()
        model = [np.float32(v) for v in np.asarray(s.model, np.float32).T.reshape(-1)]
        cloths.append((verts, idx, model, s.particle_diameter(), s.resolution, s.attached))
    sc = pyref.Scene(cloths, [pyref.collider_dict(c) for c in specs[0].colliders(0)],
                     pyref.params_dict(params_for(name)))
    xs, vs = [], []
    for _ in range(cfg["frames"]):
        sc.frame(W.FRAME_DT, cfg["substeps"], cfg["iterations"])
        xs.append(np.array(sc.x, np.float32))
        vs.append(np.array(sc.v, np.float32))
    return np.stack(xs), np.stack(vs), np.array(sc.normals(), np.float32)


def run_oracle(name, self_collision=True):
    specs, cfg = scene_specs(name), SCENES[name]
    p = params_for(name)
    p.enable_self_collision = 1 if self_collision else 0
    o = Oracle(p)
    register(o, specs)
    d = specs[-1].particle_diameter()
    xs, vs = [], []
    for _ in range(cfg["frames"]):
        o.simulate(float(W.FRAME_DT), cfg["substeps"], cfg["iterations"], 1.0, 0.1, 0.06, d)
        xs.append(o.positions())
        vs.append(o.velocities())
    return np.stack(xs), np.stack(vs), o.normals()


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_equals_python_restatement(name):
    a, b = run_oracle(name), run_pyref(name)
    for k, what in enumerate(("positions", "velocities", "normals")):
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), f"{name}: {what}"


def test_stack_scene_exercises_self_collision():
    with_sc, without = run_oracle("stack2", True), run_oracle("stack2", False)
    assert np.abs(with_sc[0][-1] - without[0][-1]).max() > 1e-3


@pytest.mark.parametrize("name", sorted(SCENES))
def test_oracle_matches_golden_fixture(name):
    g = np.load(GOLDEN / f"{name}.npz")
    x, v, n = run_oracle(name)
    assert np.array_equal(x.view(np.uint32), g["positions"].view(np.uint32))
    assert np.array_equal(v.view(np.uint32), g["velocities"].view(np.uint32))
    assert np.array_equal(n.view(np.uint32), g["normals"].view(np.uint32))
