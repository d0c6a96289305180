"""CPU: known-answer tests that pin the oracle (oracle/vt_oracle.c) independently of its
own code — answers computed here in Python from the reference formulas:

  hash        Velvet/SpatialHashGPU.cu:13-22  (int32 wrap, C remainder, abs)
  cell coord  (int)floor(x / cellSpacing) with an FP32 division
  acos        within 2 ulp of the exact arccos (the reference uses CUDA's acosf)
  constraints single stretch / attach / sphere / plane cases with analytic answers
  builder     Velvet/VtClothObjectGPU.hpp:75-147 counts and order
  free fall   PredictPositions + Finalize in FP32, step by step
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle
from oracle import Oracle
from velvet_gb300 import _abi
from velvet_gb300 import workloads as W

f32 = np.float32


def py_hash(x, y, z, table):
    def w(v):
        return v & 0xFFFFFFFF

    h = w(x * 92837111) ^ w(y * 689287499) ^ w(z * 283923481)
    if h >= 1 << 31:
        h -= 1 << 32
    r = abs(h) % table  # C's % truncates toward zero, then abs()
    return r


def test_hash_coords_known_answers():
    L = oracle.lib()
    rng = np.random.default_rng(1)
    cases = [(0, 0, 0, 7), (1, 2, 3, 8192), (-1, -1, -1, 8192), (-5, 7, -9, 131072),
             (2 ** 31 - 1, -(2 ** 31), 12345, 2097152), (46341, 46341, 46341, 13)]
    cases += [tuple(int(v) for v in rng.integers(-(2 ** 31), 2 ** 31 - 1, 3)) + (int(rng.integers(1, 1 << 22)),)
              for _ in range(2000)]
    for x, y, z, t in cases:
        assert L.vo_hash_coords(x, y, z, t) == py_hash(x, y, z, t), (x, y, z, t)


def test_direct_remainder_identity_used_by_the_neighbour_kernel():
    """The neighbour-cache kernel computes abs(h % T) as |h| mod T via
    mulhi64((M * |h|) mod 2^64, T) with M = floor((2^64 - 1) / T) + 1 (Lemire, Kaser,
    Kurz 2019); exact for all 32-bit operands."""
    rng = np.random.default_rng(9)
    ds = list(rng.integers(1, 2 ** 31 - 1, 3000)) + [1, 2, 3, 7, 8192, 131072, 2097152, 2 ** 31 - 1]
    for d in ds:
        d = int(d)
        M = ((2 ** 64 - 1) // d + 1) % 2 ** 64
        for h in list(rng.integers(-(2 ** 31), 2 ** 31 - 1, 20)) + [-(2 ** 31), -1, 0, 1, 2 ** 31 - 1]:
            h = int(h)
            n = (-h) % 2 ** 32 if h < 0 else h  # |h| as an unsigned 32-bit value
            assert ((M * n) % 2 ** 64 * d) >> 64 == py_hash_mod(h, d)


def py_hash_mod(h, table):
    r = abs(h) % table
    return r


def test_int_coord_uses_fp32_division_and_floor():
    L = oracle.lib()
    rng = np.random.default_rng(2)
    for v in list(rng.uniform(-50, 50, 3000).astype(np.float32)) + [f32(-0.0), f32(0.045), f32(-0.045)]:
        s = f32(0.045)
        want = math.floor(float(f32(v) / s))
        assert L.vo_int_coord(float(v), float(s)) == want


def test_acos_within_two_ulp():
    L = oracle.lib()
    xs = np.concatenate([np.linspace(-1, 1, 200001, dtype=np.float32),
                         np.float32(1) - np.arange(1, 2000, dtype=np.float32) * np.float32(2 ** -24),
                         np.array([0.5, -0.5, np.nextafter(np.float32(0.5), np.float32(0))], np.float32)])
    worst = 0.0
    for x in xs:
        got = f32(L.vo_acosf(float(x)))
        exact = math.acos(float(x))
        ulp = float(np.spacing(f32(exact)))
        worst = max(worst, abs(float(got) - exact) / ulp)
    assert worst <= 2.0, worst
    assert L.vo_acosf(1.0) == 0.0
    assert abs(L.vo_acosf(-1.0) - math.pi) < 4e-7


def two_particle_solver(p0, p1, **params):
    P = _abi.VtParams()
    oracle.lib().vo_params_default(C.byref(P))
    P.gravity[:] = [0.0, 0.0, 0.0]
    P.damping = 0.0
    P.enable_self_collision = 0
    for k, v in params.items():
        setattr(P, k, v)
    o = Oracle(P)
    verts = np.array([p0, p1], np.float32)
    # a large registration diameter lifts AddCloth's speed clamp (2 * d / dt * substeps)
    o.add_cloth(verts, np.zeros(0, np.uint32), np.eye(4, dtype=np.float32), 10.0)
    return o


def test_single_stretch_constraint_analytic():
    o = two_particle_solver((0, 0, 0), (2, 0, 0))
    o.add_stretch([[0, 1]], [1.0])
    o.simulate(1 / 60, 1, 1, 1.0, 0.0, 0.06, 0.001)
    x = o.positions().astype(np.float64)
    # Jacobi + averaging: each end moves (d - rest)/2 * d/(d + eps) toward the other
    move = 0.5 * (2.0 / (2.0 + 1e-6))
    assert x[0, 0] == pytest.approx(move, abs=1e-6) and x[1, 0] == pytest.approx(2 - move, abs=1e-6)
    assert np.allclose(x[:, 1:], 0)


def test_attachment_pulls_to_stretched_rest_length():
    o = two_particle_solver((0, 0, 0), (0, -3, 0))
    slot = o.add_attach_slot([0, 0, 0])
    o.add_attach([0, 1], [slot, slot], [0.0, 1.0])  # particle 0 pinned (distance 0)
    o.simulate(1 / 60, 1, 1, 1.0, 0.0, 0.06, 0.001)
    x = o.positions()
    assert o.inv_mass()[0] == 0.0
    # target = 1.0 * longRangeStretchiness (1.2): particle 1 ends at distance 1.2
    assert np.linalg.norm(x[1]) == pytest.approx(1.2, abs=1e-6)
    assert np.array_equal(x[0], np.zeros(3, np.float32))


def test_sphere_and_plane_projection():
    o = two_particle_solver((0.05, 0.1, 0), (0.5, -0.2, 0.5))
    o.update_colliders([W.sphere((0.0, 0.1, 0.0), 0.3), W.plane(0.0)])
    o.simulate(1 / 60, 1, 0, 1.0, 0.0, 0.06, 0.001)
    x = o.positions().astype(np.float64)
    # particle 0 starts inside the sphere: pushed to radius + margin (0.36) from the centre
    assert np.linalg.norm(x[0] - [0, 0.1, 0]) == pytest.approx(0.36, abs=2e-6)
    # particle 1 starts below the plane: lifted to y = margin
    assert x[1, 1] == pytest.approx(0.06, abs=1e-7)


def test_free_fall_matches_fp32_recurrence():
    P = _abi.VtParams()
    oracle.lib().vo_params_default(C.byref(P))
    P.enable_self_collision = 0
    o = Oracle(P)
    o.add_cloth(np.array([[0.0, 1.0, 0.0]], np.float32), np.zeros(0, np.uint32), np.eye(4, dtype=np.float32), 0.01)
    dt_frame, S = f32(1 / 60), 4
    dt = f32(dt_frame / f32(S))
    x, v = [f32(0), f32(1), f32(0)], [f32(0)] * 3
    g = [f32(0), f32(-9.8), f32(0)]
    for _ in range(3):
        o.simulate(float(dt_frame), S, 2, 1.0, 0.1, 0.06, 0.01)
        for _ in range(S):
            v = [v[k] + g[k] * dt for k in range(3)]
            p = [x[k] + v[k] * dt for k in range(3)]
            raw = [(p[k] - x[k]) / dt for k in range(3)]
            v = [raw[k] * (f32(1) - f32(0.25) * dt) for k in range(3)]
            x = p
    assert np.array_equal(o.positions()[0], np.array(x, np.float32))
    assert np.array_equal(o.velocities()[0], np.array(v, np.float32))


@pytest.mark.parametrize("side,nat", [(3, 2), (8, 2), (17, 17)])
def test_grid_builder_counts_and_order(side, nat):
    spec = W.ClothSpec(side, 0.02, W.horizontal_cloth(side, 0.02, 0.5), list(range(nat)),
                       W.static_colliders([]))
    o = Oracle()
    W.build_plain(spec, o)
    V = side
    si, sf = o.constraints(0)
    ai, af = o.constraints(1)
    bi, bf = o.constraints(2)
    assert sf.size == 2 * V * (V - 1) + 2 * (V - 1) ** 2
    assert bf.size == (V - 1) ** 2 and np.all(bf == 0)
    assert af.size == nat * V * V
    pairs = si.reshape(-1, 2)
    # generator (0, 0): (0,1), (0,V), (0,V+1), (1,V) (VtClothObjectGPU.hpp:90-113)
    assert pairs[:4].tolist() == [[0, 1], [0, V], [0, V + 1], [1, V]]
    assert bi.reshape(-1, 4)[0].tolist() == [0, V + 1, 1, V]
    # attachments: slot-major, every particle of the cloth per slot
    assert ai[0::2][: V * V].tolist() == list(range(V * V)) and set(ai[1::2][: V * V]) == {0}
    x = o.positions()
    assert np.array_equal(af[:V * V], np.sqrt(((x[0] - x) ** 2).sum(1, dtype=np.float32)).astype(np.float32)) \
        or np.allclose(af[:V * V], np.linalg.norm(x[0] - x, axis=1), atol=1e-6)
    w = o.inv_mass()
    assert np.all(w[:nat] == 0) and np.all(w[nat:] == 1)


def test_hash_objects_against_python_restatement():
    """Tiny table: many of the 27 neighbour cells land in the same bucket, so lists
    contain duplicates; a small per-cell cap truncates long buckets."""
    rng = np.random.default_rng(4)
    n, T, mn, sp, diam = 300, 37, 12, f32(0.1), f32(0.02)
    pos = rng.uniform(-0.3, 0.3, (n, 3)).astype(np.float32)
    orig = (pos + rng.normal(0, 0.05, (n, 3))).astype(np.float32)
    got = oracle.hash_objects(pos, orig, float(sp), T, mn, float(diam))

    coords = [tuple(math.floor(float(f32(pos[i, k]) / sp)) for k in range(3)) for i in range(n)]
    keys = [py_hash(*c, T) for c in coords]
    order = sorted(range(n), key=lambda i: (keys[i], i))
    assert got["particle_index"].tolist() == order
    assert got["particle_hash"].tolist() == [keys[i] for i in order]
    start, end = {}, {}
    for t, i in enumerate(order):
        start.setdefault(keys[i], t)
        end[keys[i]] = t + 1
    cs = got["cell_start"]
    for h in range(T):
        assert cs[h] == start.get(h, 0xFFFFFFFF)
        if h in end:
            assert got["cell_end"][h] == end[h]
    sp2, d2 = sp * sp, diam * diam

    def l2(a, b):
        d = (a - b).astype(np.float32)
        return f32(f32(d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])

    nb = got["neighbors"].reshape(mn, n)
    for i in range(n):
        want = []
        ix, iy, iz = coords[i]
        for x in (ix - 1, ix, ix + 1):
            for y in (iy - 1, iy, iy + 1):
                for z in (iz - 1, iz, iz + 1):
                    h = py_hash(x, y, z, T)
                    if h not in start:
                        continue
                    for t in range(start[h], min(end[h], start[h] + mn)):
                        j = order[t]
                        if j != i and l2(pos[i], pos[j]) < sp2 and l2(orig[i], orig[j]) > d2:
                            want.append(j)
        want = want[:mn]
        col = nb[:, i].tolist()
        assert col[: len(want)] == want
        if len(want) < mn:
            assert col[len(want)] == 0xFFFFFFFF


@pytest.mark.parametrize("res", [1, 2, 5])
def test_bending_adjacency_on_a_flat_grid(res):
    """Every interior edge of the grid mesh is a hinge: the R^2 quad diagonals the
    reference bends plus the 2R(R-1) edges between quads; flat, so every rest angle is 0."""
    verts, idx = W.grid_mesh(res, 0.02 * res)
    o = Oracle()
    off = o.add_cloth(verts, idx, np.eye(4), 0.03)
    assert o.build_bending_adjacency(off) == res * res + 2 * res * (res - 1)
    ints, rest = o.constraints(2)
    assert np.all(rest == 0.0)
    quads = ints.reshape(-1, 4)
    # the first hinge is the first quad's diagonal, with the reference's corner order
    V = res + 1
    assert quads[0].tolist() == [0, V + 1, 1, V]
    o.close()


def test_bending_adjacency_known_fold_and_non_manifold_edges():
    # two triangles folded at 90 degrees along the edge (1, 2)
    verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 1]], np.float32)
    o = Oracle()
    off = o.add_cloth(verts, np.array([0, 1, 2, 2, 1, 3], np.uint32), np.eye(4), 0.03)
    assert o.build_bending_adjacency(off) == 1
    ints, rest = o.constraints(2)
    assert ints.tolist() == [0, 3, 2, 1]
    assert abs(float(rest[0]) - math.pi / 2) < 1e-6
    o.close()
    # an edge shared by three triangles is no hinge; nor are boundary edges
    verts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.5, 0.5, 1], [0.5, 0.5, -1]], np.float32)
    o = Oracle()
    off = o.add_cloth(verts, np.array([0, 1, 2, 2, 1, 3, 1, 2, 4], np.uint32), np.eye(4), 0.03)
    assert o.build_bending_adjacency(off) == 0
    o.close()


def test_render_single_particle_known_answers():
    """The renderer's restatement: one sphere straight ahead covers a disc of the
    projected radius around the image centre, lit head-on where the light comes from
    the camera; the rest is background."""
    import velvet_gb300 as vg

    W_, H_ = 64, 48
    rp = vg.render_params(W_, H_, eye=(0, 0, 2), target=(0, 0, 0), particle_radius=0.1,
                          light_dir=(0, 0, 1), ambient=0.0, tint=(1.0, 0.5, 0.25), background=0xFF000000)
    img = oracle.render(np.zeros((1, 3), np.float32), rp)
    bg = img == 0xFF000000
    # projected radius in pixels: R * f / d * H / 2 with f = 1 / tan(22.5 deg)
    r_px = 0.1 * (1 / math.tan(math.radians(22.5))) / 2.0 * H_ / 2
    covered = int((~bg).sum())
    assert abs(covered - math.pi * r_px * r_px) < 2 * math.pi * r_px + 4
    # the pixel nearest the centre: its normal's z (the lighting term) from its offset
    j, i = H_ // 2, W_ // 2
    f = 1 / math.tan(math.radians(22.5))
    u = ((i + 0.5) / W_ * 2 - 1) / (f / (W_ / H_) / 2 * 0.1)
    v = (1 - (j + 0.5) / H_ * 2) / (f / 2 * 0.1)
    nz = math.sqrt(1 - u * u - v * v)
    c = int(img[j, i])
    for ch, tint in enumerate((1.0, 0.5, 0.25)):
        assert abs(((c >> (8 * ch)) & 0xFF) - 255 * math.sqrt(tint * nz)) <= 1.0
    assert bg[0, 0] and bg[-1, -1]
    # a nearer particle hides a farther one behind it
    two = np.array([[0, 0, 0], [0, 0, 0.5]], np.float32)
    rp.tint[:] = [1.0, 1.0, 1.0]
    img2 = oracle.render(two, rp)
    assert (img2 != 0xFF000000).sum() > covered  # the nearer sphere projects larger
