"""GPU parity: the CUDA solver against the CPU oracle on identical inputs.

Every Jacobi sum on the GPU is a per-particle gather in constraint order and all FP32
arithmetic is unfused IEEE, so the expected difference is zero: positions, velocities,
normals, hash keys, sort order, cell ranges and neighbour lists are compared bit for bit.
"""
import numpy as np
import pytest

import velvet_gb300 as vg
from velvet_gb300 import _abi
from velvet_gb300 import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def make_pair(spec, params=None):
    g, o = vg.ClothSolver(params), Oracle(params)
    for s in (g, o):
        W.build_plain(spec, s)
    return g, o


def step(wl, g, o, spec, frame, diameter):
    cols = spec.colliders(frame)
    for s in (g, o):
        s.update_colliders(cols)
        s.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                   wl.collision_margin, diameter)
    g.sync()


def assert_same(a, b, what):
    if not np.array_equal(bits(a), bits(b)):
        diff = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
        bad = np.argwhere(bits(a) != bits(b))
        raise AssertionError(f"{what}: {len(bad)} values differ, first {bad[:3].tolist()}, "
                             f"max |diff| {np.nanmax(diff):.3g}")


def small_spec(side=32, height=0.5):
    base = W.small()
    return base, W.ClothSpec(side, 0.02, W.horizontal_cloth(side, 0.02, height), [0, side - 1],
                             base.cloths[0].colliders)


def test_small_cloth_frames_bit_exact():
    wl, spec = small_spec(32, 0.45)
    g, o = make_pair(spec)
    d = spec.particle_diameter()
    for f in range(20):
        step(wl, g, o, spec, f, d)
        assert_same(g.positions(), o.positions(), f"positions frame {f}")
        assert_same(g.velocities(), o.velocities(), f"velocities frame {f}")
    assert_same(g.normals(), o.normals(), "normals")


def test_hash_views_bit_exact():
    wl, spec = small_spec(48, 0.4)
    g, o = make_pair(spec)
    d = spec.particle_diameter()
    for f in range(3):
        step(wl, g, o, spec, f, d)
    hv = o.hash_view()
    assert np.array_equal(g.debug_view(_abi.DEBUG_PARTICLE_HASH), hv["particle_hash"])
    assert np.array_equal(g.debug_view(_abi.DEBUG_PARTICLE_INDEX), hv["particle_index"])
    assert np.array_equal(g.debug_view(_abi.DEBUG_CELL_START), hv["cell_start"])
    cs = hv["cell_start"][:-1]
    occ = cs != 0xFFFFFFFF  # cellEnd is only meaningful for occupied cells
    assert np.array_equal(g.debug_view(_abi.DEBUG_CELL_END)[occ], hv["cell_end"][occ])
    n, mn = o.num_particles, o.params.max_num_neighbors
    a = g.debug_view(_abi.DEBUG_NEIGHBORS).reshape(mn, n)
    b = hv["neighbors"].reshape(mn, n)
    assert np.array_equal(valid_lists(a), valid_lists(b))
    assert (valid_lists(b) != -2).sum() > n  # lists are not empty
    assert_same(g.debug_view(_abi.DEBUG_PREDICTED), o.predicted(), "predicted")


def valid_lists(nb):
    """Column-major neighbour lists with every entry after the 0xffffffff terminator
    replaced by -2 (those slots keep stale values in the reference too)."""
    nb = nb.astype(np.int64)
    ended = np.cumsum(nb == 0xFFFFFFFF, axis=0) - (nb == 0xFFFFFFFF)
    return np.where(ended > 0, -2, nb)


def test_small_config_64_bit_exact_300_frames():
    """The small configuration for its full 300 frames (64x64, sphere + plane, 5 x 10,
    self-collision), compared bit for bit at frames 1, 30, 100 and 300."""
    wl = W.small(frames=300)
    spec = wl.cloths[0]
    g, o = make_pair(spec)
    d = spec.particle_diameter()
    for f in range(wl.frames):
        step(wl, g, o, spec, f, d)
        if f + 1 in (1, 30, 100, 300):
            assert_same(g.positions(), o.positions(), f"positions after {f + 1} frames")
            assert_same(g.velocities(), o.velocities(), f"velocities after {f + 1} frames")
    assert_same(g.normals(), o.normals(), "normals after 300 frames")
