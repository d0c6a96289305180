"""GPU: the batched solver.  Each cloth in a batch must give exactly the bits it gives
alone on the plain solver (and therefore exactly the oracle's bits): isolation of the
per-cloth hash domains, parameters and colliders, with uneven cloth sizes."""
import numpy as np
import pytest

import velvet_gb300 as vg
from velvet_gb300 import _abi
from velvet_gb300 import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def mixed(count=7, seed=3):
    return W.batched(count, frames=8, seed=seed, lo=8, hi=40)


@pytest.mark.parametrize("graphs", [True, False])
def test_batch_equals_each_cloth_alone(graphs):
    wl = mixed()
    batch = vg.BatchSolver()
    batch.use_graphs(graphs)
    alone = []
    for spec in wl.cloths:
        s = vg.ClothSolver()
        W.build_plain(spec, s)
        batch.add(s)
        o = vg.ClothSolver()
        W.build_plain(spec, o)
        alone.append((o, spec))
    for f in range(wl.frames):
        batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin)
        for o, spec in alone:
            o.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin, spec.particle_diameter())
    batch.sync()
    for k, (o, spec) in enumerate(alone):
        o.sync()
        assert np.array_equal(bits(batch.positions(k)), bits(o.positions())), f"cloth {k} positions"
        assert np.array_equal(bits(batch.velocities(k)), bits(o.velocities())), f"cloth {k} velocities"
        assert np.array_equal(bits(batch.normals(k)), bits(o.normals())), f"cloth {k} normals"


@pytest.mark.skipif(_abi.VARIANT == "fast", reason="bits of the oracle / host arithmetic: exact build only")
def test_batch_of_tiny_cloths_matches_the_oracle():
    """Five cloths of 8-16 particles a side, 2,048 particles at most in all: the whole
    hash on one block (several domains' keys, one sort, their cell ranges), the
    warp-per-particle neighbour walk and the cluster-resident substeps with the collision
    pass folded in, one cluster per cloth — each cloth the oracle's bits."""
    wl = W.batched(5, frames=6, seed=21, lo=8, hi=16)
    assert sum(c.num_particles for c in wl.cloths) <= 2048
    batch = vg.BatchSolver()
    ors = []
    for spec in wl.cloths:
        s = vg.ClothSolver()
        W.build_plain(spec, s)
        batch.add(s)
        s.close()
        o = Oracle()
        W.build_plain(spec, o)
        ors.append((o, spec))
    for f in range(wl.frames):
        batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin)
        for o, spec in ors:
            o.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin, spec.particle_diameter())
    batch.sync()
    for k, (o, spec) in enumerate(ors):
        assert np.array_equal(bits(batch.positions(k)), bits(o.positions())), f"cloth {k} positions"
        assert np.array_equal(bits(batch.velocities(k)), bits(o.velocities())), f"cloth {k} velocities"
        o.close()


def test_batch_of_more_small_cloths_than_clusters_fit_equals_each_alone():
    """64 cloths of 8-24 particles a side: more 16-block clusters than the device holds at
    once, so the batch runs one launch per Jacobi iteration while each cloth alone runs the
    cluster-resident substep — the same bits either way, and the batch's frame launches
    the tile kernel once per iteration."""
    import ctypes as C

    wl = W.batched(64, frames=3, seed=8, lo=8, hi=24)
    batch = vg.BatchSolver()
    alone = []
    for spec in wl.cloths:
        s = vg.ClothSolver()
        W.build_plain(spec, s)
        batch.add(s)
        s.close()
        o = vg.ClothSolver()
        W.build_plain(spec, o)
        alone.append((o, spec))
    for f in range(wl.frames):
        n0 = C.c_uint64()
        assert vg.lib().vt_batch_launch_count(batch.handle, C.byref(n0)) == 0
        batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin)
        n1 = C.c_uint64()
        assert vg.lib().vt_batch_launch_count(batch.handle, C.byref(n1)) == 0
        for o, spec in alone:
            o.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin, spec.particle_diameter())
    assert n1.value - n0.value >= wl.substeps * wl.iterations, "one launch per iteration"
    batch.sync()
    for k, (o, spec) in enumerate(alone):
        o.sync()
        assert np.array_equal(bits(batch.positions(k)), bits(o.positions())), f"cloth {k} positions"
        assert np.array_equal(bits(batch.velocities(k)), bits(o.velocities())), f"cloth {k} velocities"
        o.close()


def test_batch_mixing_kernel_kinds_equals_each_cloth_alone():
    """One batch holding grid cloths on the tile kernel, grid cloths on the CSR kernels
    (vt_solver_use_grid_kernel off) and a cloth whose 24 LRA slots take the slot-group
    path at a nonzero slot offset: every kind of domain in one frame, each cloth's bits
    those it has alone."""
    wl = mixed(6, seed=11)
    specs = list(wl.cloths)
    side = 24
    specs.append(W.ClothSpec(side, 0.02, W.horizontal_cloth(side, 0.02, 0.5),
                             list(range(0, side)), specs[0].colliders))
    csr = {1, 4}
    batch = vg.BatchSolver()
    alone = []
    for k, spec in enumerate(specs):
        pair = []
        for _ in range(2):
            s = vg.ClothSolver()
            W.build_plain(spec, s)
            if k in csr:
                assert vg.lib().vt_solver_use_grid_kernel(s.handle, 0) == 0
            pair.append(s)
        batch.add(pair[0])
        alone.append((pair[1], spec))
    for f in range(6):
        batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin)
        for o, spec in alone:
            o.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin, spec.particle_diameter())
    batch.sync()
    for k, (o, spec) in enumerate(alone):
        o.sync()
        assert np.array_equal(bits(batch.positions(k)), bits(o.positions())), f"cloth {k} positions"
        assert np.array_equal(bits(batch.velocities(k)), bits(o.velocities())), f"cloth {k} velocities"


@pytest.mark.skipif(_abi.VARIANT == "fast", reason="bits of the oracle / host arithmetic: exact build only")
def test_batch_matches_oracle_with_moving_collider():
    wl = mixed(3, seed=5)
    batch = vg.BatchSolver()
    ors = []
    mover = W.moving_sphere(0.2, 0.3, 1.0)
    for spec in wl.cloths:
        spec.colliders = mover
        s = vg.ClothSolver()
        W.build_plain(spec, s)
        batch.add(s)
        o = Oracle()
        W.build_plain(spec, o)
        ors.append((o, spec))
    for f in range(6):
        for k, (o, spec) in enumerate(ors):
            batch.update_colliders(k, spec.colliders(f))
            o.update_colliders(spec.colliders(f))
            o.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin, spec.particle_diameter())
        batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin)
    batch.sync()
    for k, (o, _) in enumerate(ors):
        assert np.array_equal(bits(batch.positions(k)), bits(o.positions())), f"cloth {k}"


def test_batch_launch_count_is_per_frame_not_per_cloth():
    wl = mixed(5)
    batch = vg.BatchSolver()
    for spec in wl.cloths:
        s = vg.ClothSolver()
        W.build_plain(spec, s)
        batch.add(s)
    counts = []
    for _ in range(4):
        batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction, wl.collision_margin)
        counts.append(batch.launch_count())
    batch.sync()
    per_frame = counts[3] - counts[2]
    # the second frame also times the grid kernel variants (a few extra launches, once,
    # unless an earlier world of the same size signature already did)
    assert per_frame == counts[2] - counts[1]
    assert counts[1] - counts[0] >= per_frame and counts[0] >= per_frame
    assert per_frame < 40 + 3 * wl.substeps * wl.iterations


def test_pipelined_read_back_returns_every_frame():
    """vt_batch_all_get_async: frame k's positions copy on a second stream while frame
    k+1 is enqueued; each frame's copy holds exactly that frame's state."""
    import torch

    wl = mixed(4, seed=5)

    def build():
        b = vg.BatchSolver()
        for spec in wl.cloths:
            s = vg.ClothSolver()
            W.build_plain(spec, s)
            b.add(s)
        return b

    ref, b = build(), build()
    frames = 5
    want = []
    for _ in range(frames):
        ref.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction, wl.collision_margin)
        ref.sync()
        want.append(ref.all_positions())
    n = sum(b.sizes)
    hosts = [torch.empty((n, 3), dtype=torch.float32, pin_memory=True) for _ in range(frames)]
    compute, copy = torch.cuda.Stream(), torch.cuda.Stream()
    for f in range(frames):
        b.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction, wl.collision_margin,
                   stream=compute)
        assert vg.lib().vt_batch_all_get_async(b.handle, 0, hosts[f].data_ptr(), vg.stream_handle(copy)) == 0
    copy.synchronize()
    compute.synchronize()
    for f in range(frames):
        assert np.array_equal(bits(hosts[f].numpy()), bits(want[f])), f"frame {f}"
