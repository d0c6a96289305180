"""Scenes whose results the reference's own solver kernels produced (tests/golden/ref_*.npz,
written by tests/golden/make_ref_golden.py through tests/refemu.py).  Each scene is
rebuilt here from its parameters, so the oracle (CPU) and the CUDA solver (GPU) can be run
on exactly the inputs the reference saw and compared with its outputs bit for bit.

A scene: the cloths (workloads.ClothSpec), parameter overrides, the per-frame call
arguments (substeps, iterations, relaxation, friction, margin), the frame count and the
frames after which the state was recorded.  Between them they cover the schedule's
branches (self-collision off, a hash every substep, an 8-entry neighbour cap, bending
compliance, damping, over-relaxation, no friction), every collider kind (sphere, plane,
cube, a moving sphere), long-range attachments over a whole row, and two cloths of one
solver colliding."""
from __future__ import annotations

import ctypes as C

import numpy as np

import oracle
from velvet_gb300 import _abi
from velvet_gb300 import workloads as W


def _cube():
    return W.make_collider(_abi.COLLIDER_CUBE, W.model_matrix((0.05, 0.2, 0.0), (0, 30, 10), (0.5, 0.4, 0.6)),
                           W.model_matrix((0.05, 0.2, 0.0), (0, 30, 10), (0.5, 0.4, 0.6)),
                           (0.05, 0.2, 0.0), (0.5, 0.4, 0.6))


SCENES = {
    # the small configuration's setting at 32x32: drape on a sphere + plane, 5 x 10
    "ref_small32": dict(frames=40, record=(1, 10, 20, 40), substeps=5, iterations=10, call=(1.0, 0.1, 0.06),
                        params={}),
    # a sphere moving sinusoidally (the large configuration's collider) and a cube,
    # bending compliance, heavy damping, over-relaxation, a hash every substep
    "ref_moving24": dict(frames=30, record=(1, 15, 30), substeps=4, iterations=8, call=(1.5, 0.2, 0.05),
                         params={"bend_compliance": 0.5, "damping": 1.0, "interleaved_hash": 1}),
    # the stress configuration's shape at 24x24: seeded drop height and four spheres, the
    # whole top row attached (24 LRA slots), 8 x 10
    "ref_stress24": dict(frames=16, record=(1, 8, 16), substeps=8, iterations=10, call=(1.0, 0.1, 0.06),
                         params={}),
    # two cloths of one solver: a pinned sheet and a free one falling onto it; an
    # 8-entry neighbour cap, no friction
    "ref_two_cloths": dict(frames=24, record=(1, 12, 24), substeps=3, iterations=6, call=(1.0, 0.0, 0.06),
                           params={"max_num_neighbors": 8}),
    # self-collision off, a sphere only, zero iterations in the last frames (the schedule's
    # iteration loop skipped)
    "ref_noself16": dict(frames=10, record=(1, 10), substeps=2, iterations=5, call=(1.0, 0.1, 0.06),
                         params={"enable_self_collision": 0}, zero_iterations_from=6),
}


def specs(name):
    if name == "ref_small32":
        base = W.small()
        return [W.ClothSpec(32, 0.02, W.horizontal_cloth(32, 0.02, 0.45), [0, 31], base.cloths[0].colliders)]
    if name == "ref_moving24":
        mov = W.moving_sphere(0.15, 0.2, 0.5)
        cube = _cube()
        return [W.ClothSpec(24, 0.02, W.horizontal_cloth(24, 0.02, 0.5), [0, 23],
                            lambda f: mov(f) + [cube])]
    if name == "ref_stress24":
        return W.stress(frames=16, seed=3, side=24).cloths
    if name == "ref_two_cloths":
        ground = W.static_colliders([W.sphere((0.0, 0.1, 0.0), 0.1), W.plane(0.0)])
        return [W.ClothSpec(16, 0.02, W.horizontal_cloth(16, 0.02, 0.25), [0, 15, 240, 255], ground),
                W.ClothSpec(12, 0.02, W.model_matrix((0.03, 0.32, 0.11), (90.0, 20.0, 0.0)), [], ground)]
    if name == "ref_noself16":
        return [W.ClothSpec(16, 0.03, W.horizontal_cloth(16, 0.03, 0.5), [0],
                            W.static_colliders([W.sphere((0.05, 0.25, 0.0), 0.2)]))]
    raise KeyError(name)


def params_for(name):
    p = _abi.VtParams()
    oracle.lib().vo_params_default(C.byref(p))
    for k, v in SCENES[name]["params"].items():
        setattr(p, k, v)
    return p


def register(solver, cloth_specs):
    """AddCloth + the cloth object's constraint generation, cloth after cloth."""
    for spec in cloth_specs:
        verts, idx = spec.mesh()
        off = solver.add_cloth(verts, idx, spec.model, spec.particle_diameter())
        solver.build_grid_constraints(off, spec.resolution, spec.attached)
    solver.update_colliders(cloth_specs[0].colliders(0))


def run(name, solver, on_frame=None):
    """Registers the scene on `solver` (an Oracle, RefSolver or ClothSolver) and runs it;
    returns {frame: (positions, velocities)} at the recorded frames and the final normals."""
    cfg, cl = SCENES[name], specs(name)
    register(solver, cl)
    d = cl[-1].particle_diameter()
    relax, friction, margin = cfg["call"]
    out = {}
    for f in range(cfg["frames"]):
        solver.update_colliders(cl[0].colliders(f))
        its = 0 if f >= cfg.get("zero_iterations_from", 1 << 30) else cfg["iterations"]
        solver.simulate(float(W.FRAME_DT), cfg["substeps"], its, relax, friction, margin, d)
        if hasattr(solver, "sync"):
            solver.sync()
        if f + 1 in cfg["record"]:
            out[f + 1] = (solver.positions(), solver.velocities())
        if on_frame:
            on_frame(f, solver)
    return out, solver.normals()


# HashObjects on a cloud (Velvet/SpatialHashGPU.cu:159-196): dense enough to hit the
# per-bucket and per-particle neighbour caps, a table with shared buckets
HASH_CLOUD = dict(n=3000, seed=21, half=0.12, spacing=0.045, table=4001, max_neighbors=32, diameter=0.03)


def hash_cloud_inputs():
    c = HASH_CLOUD
    rng = np.random.default_rng(c["seed"])
    pos = rng.uniform(-c["half"], c["half"], (c["n"], 3)).astype(np.float32)
    pos[:, 1] *= 0.4
    orig = (pos + rng.normal(0.0, 0.03, (c["n"], 3))).astype(np.float32)
    return pos, orig
