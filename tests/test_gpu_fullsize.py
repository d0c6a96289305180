"""GPU checks at the configurations' full sizes and shapes: the large cloth against the
oracle for 6 frames (and 60 in a slow test), a stress-shaped cloth (seeded drop height
and spheres, the whole top row attached, 8 x 10) against the oracle for 20 frames at
128x128, and size-independent properties where the oracle is too slow to follow: for the
1024x1024 stress cloth two different kernels agree bit for bit (the implicit-topology
tile kernel and the general CSR kernels) and reruns are identical; the 512-cloth mix as
one batch equals each cloth simulated alone."""

import numpy as np
import pytest

import velvet_gb300 as vg
from velvet_gb300 import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same(a, b, what):
    if not np.array_equal(bits(a), bits(b)):
        raise AssertionError(f"{what}: {(bits(a) != bits(b)).sum()} of {bits(a).size} values differ")


def frame(wl, solvers, spec, f):
    d = spec.particle_diameter()
    for s in solvers:
        s.update_colliders(spec.colliders(f))
        s.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction, wl.collision_margin, d)


def test_large_config_moving_sphere_matches_the_oracle():
    """256x256 cloth, sphere moving sinusoidally, 5 x 20: bit-exact for 6 frames."""
    wl = W.large()
    spec = wl.cloths[0]
    g, o = vg.ClothSolver(), Oracle()
    for s in (g, o):
        W.build_plain(spec, s)
    for f in range(6):
        frame(wl, (g, o), spec, f)
    g.sync()
    same(g.positions(), o.positions(), "large positions")
    same(g.velocities(), o.velocities(), "large velocities")
    same(g.normals(), o.normals(), "large normals")


@pytest.mark.slow
def test_large_config_matches_the_oracle_for_60_frames():
    """256x256 cloth, moving sphere, 5 x 20: bit-exact at frames 20, 40 and 60."""
    wl = W.large()
    spec = wl.cloths[0]
    g, o = vg.ClothSolver(), Oracle()
    for s in (g, o):
        W.build_plain(spec, s)
    for f in range(60):
        frame(wl, (g, o), spec, f)
        if (f + 1) % 20 == 0:
            g.sync()
            same(g.positions(), o.positions(), f"large positions after {f + 1} frames")
            same(g.velocities(), o.velocities(), f"large velocities after {f + 1} frames")
    same(g.normals(), o.normals(), "large normals after 60 frames")


@pytest.mark.parametrize("grid", [True, False], ids=["tile", "csr"])
def test_stress_shaped_cloth_matches_the_oracle(grid):
    """The stress configuration's shape at 128x128: drop height U(0.5, 1.5) m and four
    spheres of radius U(0.1, 0.4) m from seed 0, plane, the whole top row attached (128
    LRA slots: eight slot groups of 16 in two super-groups, the tile kernel's group
    skips), 8 substeps x 10 iterations, bit-exact against the oracle at frames 1, 5, 10,
    15 and 20, through the tile kernel and through the CSR kernels."""
    wl = W.stress(frames=20, seed=0, side=128)
    spec = wl.cloths[0]
    g, o = vg.ClothSolver(), Oracle()
    for s in (g, o):
        W.build_plain(spec, s)
    assert vg.lib().vt_solver_use_grid_kernel(g.handle, 1 if grid else 0) == 0
    moved = 0.0
    x0 = o.positions()
    for f in range(wl.frames):
        frame(wl, (g, o), spec, f)
        if f + 1 in (1, 5, 10, 15, 20):
            g.sync()
            same(g.positions(), o.positions(), f"stress-shaped positions after {f + 1} frames")
            same(g.velocities(), o.velocities(), f"stress-shaped velocities after {f + 1} frames")
            moved = float(np.abs(o.positions() - x0).max())
    same(g.normals(), o.normals(), "stress-shaped normals after 20 frames")
    assert moved > 0.1, "the cloth should have fallen"


def test_stress_config_tile_and_csr_kernels_agree_and_rerun_identically():
    """1024x1024 cloth with the whole top row attached (1,024 LRA slots), 8 x 10: the tile
    kernel, the CSR kernels and a second tile-kernel run give the same bits."""
    wl = W.stress()
    spec = wl.cloths[0]
    runs = []
    for grid in (True, False, True):
        s = vg.ClothSolver()
        W.build_plain(spec, s)
        assert vg.lib().vt_solver_use_grid_kernel(s.handle, 1 if grid else 0) == 0
        frame(wl, (s,), spec, 0)
        s.sync()
        runs.append((s.positions(), s.velocities()))
        s.close()
    for k, what in ((1, "CSR kernels"), (2, "rerun")):
        same(runs[k][0], runs[0][0], f"stress positions, {what}")
        same(runs[k][1], runs[0][1], f"stress velocities, {what}")


def test_batched_mix_full_size_equals_each_cloth_alone():
    """The bench's 512-cloth mix (6.9 M particles): two frames as one batch equal every
    cloth's two frames on its own solver."""
    wl = W.batched()
    batch, alone = vg.BatchSolver(), []
    for spec in wl.cloths:
        s = vg.ClothSolver()
        W.build_plain(spec, s)
        batch.add(s)
        alone.append(s)
    for f in range(2):
        batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction, wl.collision_margin)
        for s, spec in zip(alone, wl.cloths):
            frame(wl, (s,), spec, f)
    batch.sync()
    got = batch.all_positions()
    want = np.concatenate([s.positions() for s in alone])
    same(got, want, "batched mix positions")
