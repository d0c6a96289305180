"""GPU parity beyond the default configuration: the generic (CSR) constraint path and the
implicit-topology grid path against each other and the oracle, and the branches of the
reference schedule and API that the benchmark configs do not take.  Every comparison is
bit-exact (see tests/test_gpu_parity.py)."""
import math

import numpy as np
import pytest

import velvet_gb300 as vg
from velvet_gb300 import _abi
from velvet_gb300 import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same(a, b, what):
    if not np.array_equal(bits(a), bits(b)):
        d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
        raise AssertionError(f"{what}: {(bits(a) != bits(b)).sum()} values differ, max {np.nanmax(d):.3g}")


def spec_of(side=20, height=0.45, attached=None, colliders=None):
    base = W.small()
    return W.ClothSpec(side, 0.02, W.horizontal_cloth(side, 0.02, height),
                       [0, side - 1] if attached is None else attached,
                       colliders or base.cloths[0].colliders)


def run_frames(solvers, spec, frames, substeps=5, iterations=10, relax=1.0, friction=0.1, margin=0.06,
               frame_hook=None):
    d = spec.particle_diameter()
    for f in range(frames):
        if frame_hook:
            frame_hook(f)
        for s in solvers:
            s.update_colliders(spec.colliders(f))
            s.simulate(float(W.FRAME_DT), substeps, iterations, relax, friction, margin, d)
    for s in solvers:
        if isinstance(s, vg.ClothSolver):
            s.sync()


def generic_copy(spec, o: Oracle, params=None):
    """A GPU solver registered through AddStretch / AddAttachSlot / AddAttach / AddBend
    with exactly the constraints the oracle's builder made: the CSR path."""
    g = vg.ClothSolver(params)
    verts, idx = spec.mesh()
    g.add_cloth(verts, idx, spec.model, spec.particle_diameter())
    si, sf = o.constraints(0)
    g.add_stretch(si.reshape(-1, 2), sf)
    pos = o.positions()
    for p in spec.attached:
        g.add_attach_slot(pos[p])
    ai, af = o.constraints(1)
    if af.size:
        g.add_attach(ai[0::2], ai[1::2], af)
    bi, bf = o.constraints(2)
    g.add_bend(bi.reshape(-1, 4), bf)
    g.update_colliders(spec.colliders(0))
    return g


def test_csr_path_grid_path_and_oracle_agree():
    spec = spec_of(22)
    o = Oracle()
    W.build_plain(spec, o)
    csr = generic_copy(spec, o)
    grid = vg.ClothSolver()
    W.build_plain(spec, grid)
    run_frames([o, csr, grid], spec, 12)
    same(csr.positions(), o.positions(), "csr vs oracle")
    same(grid.positions(), o.positions(), "grid vs oracle")
    same(grid.normals(), csr.normals(), "normals grid vs csr")


@pytest.mark.parametrize("tile_edge", [6, 7, 8, 31, 32, 33, 40])
def test_grid_tiles_at_every_edge_case(tile_edge):
    """Cloth sides around the 7 x 31 tile shape: partial tiles on both axes."""
    spec = spec_of(tile_edge, 0.4)
    o = Oracle()
    W.build_plain(spec, o)
    g = vg.ClothSolver()
    W.build_plain(spec, g)
    run_frames([o, g], spec, 4)
    same(g.positions(), o.positions(), f"side {tile_edge}")
    same(g.velocities(), o.velocities(), f"side {tile_edge} velocities")


@pytest.mark.parametrize("side", [37, 64])
@pytest.mark.parametrize("variant", range(len(vg.GRID_VARIANTS)))
def test_every_grid_tile_shape_gives_the_same_bits(variant, side):
    """The autotuner chooses among tile shapes and occupancies; each must reproduce the
    oracle exactly.  Sides of 37 and 64 vertices leave partial tiles for every shape (64:
    a last row of tiles one particle high for 7x31 and 3x63, a last column one wide for
    3x63)."""
    import ctypes as C

    assert vg.lib().vt_tuning_set_grid_tile(variant) == 0
    try:
        spec = spec_of(side, 0.4)
        o, g = Oracle(), vg.ClothSolver()
        for s in (o, g):
            W.build_plain(spec, s)
        run_frames([o, g], spec, 4)
        same(g.positions(), o.positions(), f"tile shape {variant}, side {side}")
        same(g.velocities(), o.velocities(), f"tile shape {variant}, side {side} velocities")
        used = C.c_int32()
        assert vg.lib().vt_solver_grid_tile(g.handle, C.byref(used)) == 0 and used.value == variant
    finally:
        vg.lib().vt_tuning_set_grid_tile(-1)


@pytest.mark.parametrize("tma", [1, 0], ids=["tma", "cp_async"])
@pytest.mark.parametrize("variant", [0, 2, 4])
def test_tile_loads_by_tma_and_by_cp_async_give_the_oracle_bits(variant, tma):
    """The tile kernel stages its halo, rests and positions with TMA bulk tensor copies
    or per-thread cp.async (the default; vt_tuning_set_tile_loads): both give the oracle's
    bits, for every tile shape, on a cloth with partial tiles, two cached LRA slots and
    the finalizing iterations' position loads, and on a batch of cloths of several sizes."""
    assert vg.lib().vt_tuning_set_tile_loads(tma) == 0
    assert vg.lib().vt_tuning_set_grid_tile(variant) == 0
    try:
        spec = spec_of(45, 0.4)
        o, g = Oracle(), vg.ClothSolver()
        for s in (o, g):
            W.build_plain(spec, s)
        run_frames([o, g], spec, 3)
        same(g.positions(), o.positions(), f"tile loads {tma}, shape {variant}")
        same(g.velocities(), o.velocities(), f"tile loads {tma}, shape {variant} velocities")
        wl = W.batched(5, frames=2, seed=9, lo=10, hi=70)
        batch, alone = vg.BatchSolver(), []
        for c in wl.cloths:
            s = vg.ClothSolver()
            W.build_plain(c, s)
            batch.add(s)
            s.close()
            a = Oracle()
            W.build_plain(c, a)
            alone.append(a)
        for f in range(wl.frames):
            batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction, wl.collision_margin)
            for a, c in zip(alone, wl.cloths):
                a.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                           wl.collision_margin, c.particle_diameter())
        batch.sync()
        for k, a in enumerate(alone):
            same(batch.positions(k), a.positions(), f"tile loads {tma}, batch cloth {k}")
    finally:
        vg.lib().vt_tuning_set_grid_tile(-1)
        vg.lib().vt_tuning_set_tile_loads(0)


@pytest.mark.parametrize("clusters", [1, 2, 0], ids=["resident", "clusters", "per_iteration"])
@pytest.mark.parametrize("variant", [0, 1, 2])
def test_substeps_in_clusters_give_the_oracle_bits(variant, clusters):
    """Small grid cloths run a substep's iterations as one launch of 16-block clusters,
    one per cloth, with the cluster barrier between iterations: positions resident in the
    blocks' shared memory with halos passed through distributed shared memory (mode 1),
    or re-read from global memory each iteration (mode 2), or one launch per iteration
    (mode 0).  The oracle's bits in every mode: a 40x40 cloth (9 to 14 tiles, one per
    block, for the three shapes; 3x3 resident tiles with partial edges), a 24x24 one
    (fewer tiles than blocks), a 64x64 one (4x4 full resident tiles; two rounds of tiles in
    mode 2 are not taken, so per-iteration launches), a 17x17 one with its whole top row
    attached (more slots than the tile caches: the slot-group boxes), odd and even
    iteration counts, the finalizing iterations between substeps, and a batch of small
    cloths."""
    assert vg.lib().vt_tuning_set_substep_clusters(clusters) == 0
    assert vg.lib().vt_tuning_set_grid_tile(variant) == 0
    try:
        for side, its, attached in ((40, 10, None), (24, 3, None), (64, 10, None), (17, 4, list(range(17)))):
            spec = spec_of(side, 0.45, attached=attached)
            o, g = Oracle(), vg.ClothSolver()
            for s in (o, g):
                W.build_plain(spec, s)
            run_frames([o, g], spec, 3, substeps=3, iterations=its)
            same(g.positions(), o.positions(), f"clusters {clusters}, shape {variant}, side {side}")
            same(g.velocities(), o.velocities(), f"clusters {clusters}, shape {variant}, side {side} velocities")
        wl = W.batched(6, frames=2, seed=4, lo=8, hi=44)
        batch, alone = vg.BatchSolver(), []
        for c in wl.cloths:
            s = vg.ClothSolver()
            W.build_plain(c, s)
            batch.add(s)
            s.close()
            a = Oracle()
            W.build_plain(c, a)
            alone.append(a)
        for f in range(wl.frames):
            batch.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction, wl.collision_margin)
            for a, c in zip(alone, wl.cloths):
                a.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                           wl.collision_margin, c.particle_diameter())
        batch.sync()
        for k, a in enumerate(alone):
            same(batch.positions(k), a.positions(), f"clusters {clusters}, batch cloth {k}")
    finally:
        vg.lib().vt_tuning_set_grid_tile(-1)
        vg.lib().vt_tuning_set_substep_clusters(1)


def test_substep_cluster_mode_out_of_range_is_refused():
    assert vg.lib().vt_tuning_set_substep_clusters(3) != 0
    assert vg.lib().vt_tuning_set_substep_clusters(-1) != 0
    assert vg.lib().vt_tuning_set_substep_clusters(1) == 0


def test_substeps_in_clusters_cut_the_launches_of_a_small_cloth():
    """With clusters, a 32x32 cloth's frame launches one grid kernel per substep instead of
    one per iteration."""
    import ctypes as C

    counts = {}
    for clusters in (1, 2, 0):
        assert vg.lib().vt_tuning_set_substep_clusters(clusters) == 0
        try:
            spec = spec_of(32, 0.45)
            g = vg.ClothSolver()
            W.build_plain(spec, g)
            run_frames([g], spec, 3, substeps=5, iterations=10)  # past the autotuner's frame
            n0 = C.c_uint64()
            assert vg.lib().vt_solver_launch_count(g.handle, C.byref(n0)) == 0
            run_frames([g], spec, 1, substeps=5, iterations=10)
            n1 = C.c_uint64()
            assert vg.lib().vt_solver_launch_count(g.handle, C.byref(n1)) == 0
            counts[clusters] = n1.value - n0.value
        finally:
            vg.lib().vt_tuning_set_substep_clusters(1)
    assert counts[0] - counts[1] == 5 * (10 - 1), counts
    assert counts[2] == counts[1], counts


@pytest.mark.parametrize("variant", [-1, 1, 5])
@pytest.mark.parametrize("n_slots", [5, 24])
def test_many_lra_slots_recompute_their_rests(n_slots, variant):
    """More attach slots than the per-particle cache holds (the stress configuration
    attaches a whole row): the tile kernel recomputes |slot0 - x0| for each slot, at four
    and at five resident blocks per SM."""
    assert vg.lib().vt_tuning_set_grid_tile(variant) == 0
    try:
        side = 24
        spec = spec_of(side, 0.4, attached=list(range(0, side, side // n_slots))[:n_slots])
        o, g = Oracle(), vg.ClothSolver()
        for s in (o, g):
            W.build_plain(spec, s)
        run_frames([o, g], spec, 5)
        same(g.positions(), o.positions(), f"{n_slots} LRA slots")
        same(g.velocities(), o.velocities(), f"{n_slots} LRA slots velocities")
    finally:
        vg.lib().vt_tuning_set_grid_tile(-1)


@pytest.mark.parametrize("n_slots", [2, 24])
def test_lra_at_stretchiness_one_keeps_every_boundary_pair_exact(n_slots):
    """Long-range stretchiness 1.0: every LRA pair starts at its target distance, so the
    squared-distance filter that lets a pair skip its square roots sees pairs on both
    sides of its bound and just inside it for the whole run; the cached (2 slots) and
    recomputed (24 slots) forms must stay bit-exact with the oracle."""
    side = 24
    attached = [0, side - 1] if n_slots == 2 else list(range(0, side, side // n_slots))[:n_slots]
    spec = spec_of(side, 0.4, attached=attached)
    p = vg.default_params()
    p.long_range_stretchiness = 1.0
    o, g = Oracle(params=p), vg.ClothSolver(p)
    for s in (o, g):
        W.build_plain(spec, s)
    run_frames([o, g], spec, 6)
    same(g.positions(), o.positions(), f"{n_slots} LRA slots at stretchiness 1")
    same(g.velocities(), o.velocities(), f"{n_slots} LRA slots at stretchiness 1, velocities")


@pytest.mark.parametrize("lrs", [1.2, 1.0])
@pytest.mark.parametrize("side,rows", [(64, 1), (40, 30)])
def test_lra_slot_groups_skip_only_quiet_groups(side, rows, lrs):
    """Whole attached rows (64 slots: four groups of 16; 1,200 slots: 64 groups of 19, the
    last of 3): the tile kernel skips a group of slots when bounding boxes prove none of
    its pairs fires.  Stretchiness 1.0 puts pairs at their bound; the result must be the
    oracle's."""
    spec = spec_of(side, 0.4, attached=list(range(rows * side)))
    p = vg.default_params()
    p.long_range_stretchiness = lrs
    o, g = Oracle(params=p), vg.ClothSolver(p)
    for s in (o, g):
        W.build_plain(spec, s)
    run_frames([o, g], spec, 3 if rows > 1 else 6)
    same(g.positions(), o.positions(), f"{rows * side} slots, stretchiness {lrs}")
    same(g.velocities(), o.velocities(), f"{rows * side} slots, stretchiness {lrs}, velocities")


def test_moving_slots_keep_group_bounds_exact():
    """A whole attached row (40 slots: groups of 16) dragged sideways and up frame by frame:
    the slot groups' boxes are rebuilt from the current slot positions every iteration,
    so skipping a group stays exact while the slots move."""
    side = 40
    spec = spec_of(side, 0.4, attached=list(range(side)))
    o, g = Oracle(), vg.ClothSolver()
    for s in (o, g):
        W.build_plain(spec, s)
    start = o.positions()[:side].copy()

    def hook(f):
        shift = np.array([0.03 * f, 0.01 * f, -0.02 * f], np.float32)
        for s in (o, g):
            for k in range(side):
                s.set_attach_slot(k, start[k] + shift)

    run_frames([o, g], spec, 6, frame_hook=hook)
    same(g.positions(), o.positions(), "dragged row positions")
    same(g.velocities(), o.velocities(), "dragged row velocities")


def checkerboard_mesh(res, size):
    """A grid whose quad diagonals alternate direction: not the reference's mesh."""
    verts, _ = W.grid_mesh(res, size)
    V = res + 1
    tris = []
    for a in range(res):
        for b in range(res):
            p, q, r, s = a * V + b, (a + 1) * V + b, a * V + b + 1, (a + 1) * V + b + 1
            tris += [p, q, r, r, q, s] if (a + b) % 2 == 0 else [p, q, s, p, s, r]
    return verts, np.array(tris, np.uint32)


def unique_edges(idx):
    e = set()
    for t in idx.reshape(-1, 3):
        for k in range(3):
            u, v = int(t[k]), int(t[(k + 1) % 3])
            e.add((min(u, v), max(u, v)))
    return np.array(sorted(e), np.int32)


@pytest.mark.parametrize("mesh", ["grid", "checkerboard"])
def test_general_bending_adjacency_matches_the_oracle(mesh):
    """vt_cloth_build_bending_adjacency (a hinge per interior edge, rest angle measured at
    the initial shape) built by the library and by the oracle, solved by the CSR kernels."""
    res = 14
    spec = spec_of(res + 1, 0.5)
    if mesh == "grid":
        verts, idx = spec.mesh()
    else:
        verts, idx = checkerboard_mesh(res, 0.02 * res)
    o, g = Oracle(), vg.ClothSolver()
    counts = []
    for s in (o, g):
        off = s.add_cloth(verts, idx, spec.model, spec.particle_diameter())
        if mesh == "grid":
            s.build_grid_constraints(off, res, spec.attached)
        else:
            e = unique_edges(idx)
            x0 = s.positions()
            rest = np.sqrt(((x0[e[:, 0]] - x0[e[:, 1]]).astype(np.float32) ** 2).sum(1)).astype(np.float32)
            s.add_stretch(e, rest)
        counts.append(s.build_bending_adjacency(off))
        s.update_colliders(spec.colliders(0))
    assert counts[0] == counts[1] == res * res + 2 * res * (res - 1)
    run_frames([o, g], spec, 6)
    same(g.positions(), o.positions(), f"{mesh} + adjacency bending")
    same(g.velocities(), o.velocities(), f"{mesh} + adjacency bending velocities")


@pytest.mark.parametrize("case", ["no_self_collision", "zero_iterations", "hash_every_substep",
                                  "bend_compliance", "no_friction", "relaxation", "max_neighbors_8",
                                  "max_speed_clamp", "no_damping", "heavy_damping", "hash_cells_larger"])
def test_schedule_branches(case):
    p = vg.default_params()
    kw = {}
    if case == "no_self_collision":
        p.enable_self_collision = 0
    elif case == "zero_iterations":
        kw["iterations"] = 0
    elif case == "hash_every_substep":
        p.interleaved_hash = 1
    elif case == "bend_compliance":
        p.bend_compliance = 0.5
    elif case == "no_friction":
        kw["friction"] = 0.0
    elif case == "relaxation":
        kw["relax"] = 1.4
    elif case == "max_neighbors_8":
        p.max_num_neighbors = 8
    elif case == "no_damping":
        p.damping = 0.0
    elif case == "heavy_damping":
        p.damping = 20.0
    elif case == "hash_cells_larger":  # more candidates per bucket, more per-bucket truncation
        p.hash_cell_size_scalar = 3.0
    spec = spec_of(18, 0.35)
    o, g = Oracle(p), vg.ClothSolver(p)
    for s in (o, g):
        W.build_plain(spec, s)
        if case == "max_speed_clamp":  # AddCloth sets maxSpeed; lowered after it so Finalize clamps
            q = s.params
            q.max_speed = 0.4
            s.params = q
    run_frames([o, g], spec, 6, **kw)
    same(g.positions(), o.positions(), case)
    same(g.velocities(), o.velocities(), case + " velocities")


def test_two_cloths_in_one_solver_collide_like_the_reference():
    """Several cloths in one plain solver share one hash and collide with each other
    (VtClothSolverGPU::AddCloth merges them); the second cloth uses the CSR path."""
    a = spec_of(16, 0.5)
    b = spec_of(16, 0.53)
    o, g = Oracle(), vg.ClothSolver()
    for s in (o, g):
        W.build_plain(a, s)
        verts, idx = b.mesh()
        off = s.add_cloth(verts, idx, b.model, b.particle_diameter())
        s.build_grid_constraints(off, b.resolution, b.attached)
        s.update_colliders(a.colliders(0))
    run_frames([o, g], a, 8)
    same(g.positions(), o.positions(), "merged cloths")
    hv = o.hash_view()
    assert np.array_equal(g.debug_view(_abi.DEBUG_PARTICLE_INDEX), hv["particle_index"])


def test_cube_collider_and_moving_slot_and_grabber_edits():
    cube = W.make_collider(_abi.COLLIDER_CUBE, W.model_matrix((0.05, 0.2, 0.0), (0, 30, 10), (0.5, 0.4, 0.6)),
                           W.model_matrix((0.0, 0.2, 0.0), (0, 25, 10), (0.5, 0.4, 0.6)),
                           (0.05, 0.2, 0.0), (0.5, 0.4, 0.6))
    spec = spec_of(20, 0.5, colliders=W.static_colliders([cube, W.plane(0.0)]))
    o, g = Oracle(), vg.ClothSolver()
    for s in (o, g):
        W.build_plain(spec, s)
    n = spec.num_particles

    def hook(f):
        if f == 2:  # MouseGrabber: pin a particle and drag it (Velvet/MouseGrabber.hpp:45-76)
            for s in (o, g):
                w = np.zeros(1, np.float32)
                s.set_inv_mass(w, first=n // 2)
                xyz = s.positions()[n // 2] + np.float32(0.01)
                s.set_positions(xyz.reshape(1, 3), first=n // 2)
        if f >= 3:  # swirl scene: move attach slot 0 (Velvet/main.cpp:326-331)
            t = f * float(W.FRAME_DT) * 3
            pos = np.array([math.sin(t) * 0.1, 0.6, 0.2], np.float32)
            for s in (o, g):
                s.set_attach_slot(0, pos)

    run_frames([o, g], spec, 7, frame_hook=hook)
    same(g.positions(), o.positions(), "cube + grabber + slot")
    same(g.inv_mass(), o.inv_mass(), "inverse masses")


def test_state_round_trip_and_numeric_fault_flag():
    spec = spec_of(12, 0.4)
    g = vg.ClothSolver()
    W.build_plain(spec, g)
    run_frames([g], spec, 2)
    x = g.positions()
    g.set_positions(x)
    same(g.positions(), x, "positions round trip")
    v = g.velocities()
    v[5] = np.nan  # a NaN injected on the host must be reported, not crash
    g.set_velocities(v)
    g.simulate(float(W.FRAME_DT), 2, 2, 1.0, 0.1, 0.06, spec.particle_diameter())
    with pytest.raises(vg.VtError) as e:
        g.sync()
    assert e.value.status == _abi.VT_ERR_NUMERIC
    g.sync()  # the flag is cleared once reported


def test_checkpoint_resume_continues_bit_for_bit():
    """vt_solver_state_save after some frames, load into a solver registered the same way:
    the resumed run equals the uninterrupted one, moving slot and grabbed particle included."""
    spec = spec_of(20, 0.5)
    a = vg.ClothSolver()
    W.build_plain(spec, a)
    run_frames([a], spec, 4)
    a.set_attach_slot(0, np.array([0.05, 0.62, 0.2], np.float32))
    w = a.inv_mass()
    w[33] = 0.0
    a.set_inv_mass(w)
    state = a.save_state()
    b = vg.ClothSolver()
    W.build_plain(spec, b)
    b.load_state(state)
    for f in range(4, 9):
        for s in (a, b):
            s.update_colliders(spec.colliders(f))
            s.simulate(float(W.FRAME_DT), 5, 10, 1.0, 0.1, 0.06, spec.particle_diameter())
    a.sync()
    b.sync()
    same(b.positions(), a.positions(), "resumed positions")
    same(b.velocities(), a.velocities(), "resumed velocities")
    other = vg.ClothSolver()
    W.build_plain(spec_of(12, 0.5), other)
    with pytest.raises(vg.VtError):
        other.load_state(state)  # another particle count
