"""Synthetic cloth workloads: grid meshes, transforms, colliders and the benchmark
configurations (small / large / stress / batched / serving).

Geometry follows the reference's scene helpers:
  grid mesh        Scene::GenerateClothMesh (Velvet/Scene.hpp:131-168), with the cloth
                   size set to spacing * resolution instead of the fixed 2 m
  model matrix     Transform::matrix (Velvet/Transform.hpp:22-29): T * Ry * Rz * Rx * S
                   (Helper::RotateWithDegree, Velvet/Helper.cpp:8-15)
  colliders        Collider (Velvet/Collider.hpp:25-41) + UpdateColliders
                   (Velvet/VtClothSolverGPU.hpp:187-205)
  diameter         |v0 - v1| * particleDiameterScalar (Velvet/VtClothObjectGPU.hpp:49)
All random draws use numpy's PCG64 generator seeded with the config's seed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable

import numpy as np

from ._abi import COLLIDER_PLANE, COLLIDER_SPHERE, VtSdfCollider

FRAME_DT = np.float32(1.0 / 60.0)  # Timer::m_fixedDeltaTime, Velvet/Timer.hpp:235


def grid_mesh(resolution: int, cloth_size: float) -> tuple[np.ndarray, np.ndarray]:
    """(resolution+1)^2 vertices and 2*resolution^2 triangles in GenerateClothMesh order."""
    r = np.float32(resolution)
    V = resolution + 1
    ys, xs = np.meshgrid(np.arange(V, dtype=np.float32), np.arange(V, dtype=np.float32), indexing="ij")
    fx = xs.reshape(-1) / r - np.float32(0.5)
    fy = -(ys.reshape(-1) / r)
    size = np.float32(cloth_size)
    verts = np.stack([size * fx, size * fy, np.zeros_like(fx)], axis=1).astype(np.float32)
    a, b = np.meshgrid(np.arange(resolution), np.arange(resolution), indexing="ij")
    a = a.reshape(-1).astype(np.int64)
    b = b.reshape(-1).astype(np.int64)
    vat = lambda x, y: x * V + y  # noqa: E731 — VertexIndexAt(x, y)
    idx = np.stack([vat(a, b), vat(a + 1, b), vat(a, b + 1),
                    vat(a, b + 1), vat(a + 1, b), vat(a + 1, b + 1)], axis=1)
    return verts, idx.reshape(-1).astype(np.uint32)


def _rot(axis: str, deg: float) -> np.ndarray:
    t = math.radians(deg)
    c, s = math.cos(t), math.sin(t)
    m = np.eye(4)
    if axis == "x":
        m[1, 1], m[1, 2], m[2, 1], m[2, 2] = c, -s, s, c
    elif axis == "y":
        m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    else:
        m[0, 0], m[0, 1], m[1, 0], m[1, 1] = c, -s, s, c
    return m


def model_matrix(position=(0.0, 0.0, 0.0), rotation_deg=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Transform::matrix: translate * rotY * rotZ * rotX * scale, float32."""
    t = np.eye(4)
    t[:3, 3] = position
    s = np.diag([scale[0], scale[1], scale[2], 1.0])
    m = t @ _rot("y", rotation_deg[1]) @ _rot("z", rotation_deg[2]) @ _rot("x", rotation_deg[0]) @ s
    return m.astype(np.float32)


def _colmajor(m: np.ndarray) -> list[float]:
    return list(np.ascontiguousarray(np.asarray(m, np.float32).T).reshape(-1))


def make_collider(kind: int, cur: np.ndarray, last: np.ndarray, position, scale,
                  delta_time: float = float(FRAME_DT)) -> VtSdfCollider:
    c = VtSdfCollider()
    c.type = kind
    c.position[:] = [float(v) for v in position]
    c.scale[:] = [float(v) for v in scale]
    c.delta_time = float(np.float32(delta_time))
    c.cur_transform[:] = _colmajor(np.asarray(cur, np.float32)[:3, :3])
    inv = np.linalg.inv(np.asarray(cur, np.float64)).astype(np.float32)
    c.inv_cur_transform[:] = _colmajor(inv)
    c.last_transform[:] = _colmajor(last)
    return c


def sphere(center, radius: float, last_center=None) -> VtSdfCollider:
    cur = model_matrix(center, (0, 0, 0), (radius, radius, radius))
    last = cur if last_center is None else model_matrix(last_center, (0, 0, 0), (radius, radius, radius))
    return make_collider(COLLIDER_SPHERE, cur, last, center, (radius, radius, radius))


def plane(height: float = 0.0) -> VtSdfCollider:
    cur = model_matrix((0.0, height, 0.0))
    return make_collider(COLLIDER_PLANE, cur, cur, (0.0, height, 0.0), (1.0, 1.0, 1.0))


@dataclass
class ClothSpec:
    """One grid cloth: vertices per side, spacing, placement, pinned vertices, colliders."""

    side: int
    spacing: float
    model: np.ndarray
    attached: list[int]
    colliders: Callable[[int], list[VtSdfCollider]]  # frame index -> collider list

    @property
    def resolution(self) -> int:
        return self.side - 1

    @property
    def num_particles(self) -> int:
        return self.side * self.side

    def mesh(self) -> tuple[np.ndarray, np.ndarray]:
        return grid_mesh(self.resolution, self.spacing * self.resolution)

    def particle_diameter(self, scalar: float = 1.5) -> float:
        """|v0 - v1| * scalar on the untransformed mesh, in FP32 with glm's dot order."""
        v, _ = self.mesh()
        d = (v[0] - v[1]).astype(np.float32)
        length = np.sqrt(np.float32(np.float32(d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]))
        return float(np.float32(length) * np.float32(scalar))


@dataclass
class Workload:
    name: str
    cloths: list[ClothSpec]
    substeps: int
    iterations: int
    frames: int
    relaxation: float = 1.0
    friction: float = 0.1
    collision_margin: float = 0.06
    frame_dt: float = float(FRAME_DT)
    seed: int = 0
    notes: dict = field(default_factory=dict)

    @property
    def num_particles(self) -> int:
        return sum(c.num_particles for c in self.cloths)


def horizontal_cloth(side: int, spacing: float, height: float) -> np.ndarray:
    """Model matrix laying the grid flat at `height`, centred on the origin, its first
    row (the 'top' edge, vertex indices 0..side-1) at z = +size/2."""
    size = spacing * (side - 1)
    return model_matrix((0.0, height, size / 2.0), (90.0, 0.0, 0.0))


def static_colliders(cols: list[VtSdfCollider]) -> Callable[[int], list[VtSdfCollider]]:
    return lambda frame: cols


def moving_sphere(radius: float, amplitude: float, hz: float, height: float | None = None):
    """Sphere oscillating along x (amplitude m, hz), last/current transforms per frame."""
    y = radius if height is None else height

    def at(frame: int):
        t = frame * float(FRAME_DT)
        return (amplitude * math.sin(2 * math.pi * hz * t), y, 0.0)

    def cols(frame: int):
        cur = at(frame)
        last = at(frame - 1) if frame > 0 else cur
        return [sphere(cur, radius, last), plane(0.0)]

    return cols


def small(frames: int = 300) -> Workload:
    """64x64 grid (4,096 particles), spacing 0.02 m, two top corners pinned, sphere
    r = 0.3 m + ground plane, 5 substeps x 10 iterations, self-collision on."""
    side = 64
    spec = ClothSpec(side, 0.02, horizontal_cloth(side, 0.02, 0.8), [0, side - 1],
                     static_colliders([sphere((0.0, 0.3, 0.0), 0.3), plane(0.0)]))
    return Workload("small_64x64", [spec], 5, 10, frames)


def large(frames: int = 600) -> Workload:
    """256x256 grid (65,536 particles), sphere r = 0.3 m moving sinusoidally
    (0.5 m, 0.5 Hz) + plane, 5 substeps x 20 iterations."""
    side = 256
    spec = ClothSpec(side, 0.02, horizontal_cloth(side, 0.02, 1.0), [0, side - 1],
                     moving_sphere(0.3, 0.5, 0.5))
    return Workload("large_256x256", [spec], 5, 20, frames)


def stress(frames: int = 120, seed: int = 0, side: int = 1024) -> Workload:
    """1024x1024 grid (1,048,576 particles), drop height U(0.5, 1.5) m, 4 spheres with
    radii U(0.1, 0.4) m + plane, the whole top row attached (1,024 slots),
    8 substeps x 10 iterations."""
    rng = np.random.default_rng(seed)
    h = float(rng.uniform(0.5, 1.5))
    size = 0.02 * (side - 1)
    cols = []
    for _ in range(4):
        r = float(rng.uniform(0.1, 0.4))
        cx, cz = (float(v) for v in rng.uniform(-size / 2, size / 2, 2))
        cols.append(sphere((cx, r, cz), r))
    cols.append(plane(0.0))
    spec = ClothSpec(side, 0.02, horizontal_cloth(side, 0.02, h), list(range(side)),
                     static_colliders(cols))
    return Workload(f"stress_{side}x{side}", [spec], 8, 10, frames, seed=seed)


def batched(count: int = 512, frames: int = 300, seed: int = 0, lo: int = 16, hi: int = 256) -> Workload:
    """`count` independent cloths, side log-uniform in [lo, hi] (round(exp(U(ln lo,
    ln hi)))), each with its own sphere (r = 0.3 m) + plane and two pinned corners,
    5 substeps x 10 iterations."""
    rng = np.random.default_rng(seed)
    sides = np.rint(np.exp(rng.uniform(math.log(lo), math.log(hi), count))).astype(int)
    cloths = []
    for s in sides:
        s = int(s)
        cloths.append(ClothSpec(s, 0.02, horizontal_cloth(s, 0.02, 0.8), [0, s - 1],
                                static_colliders([sphere((0.0, 0.3, 0.0), 0.3), plane(0.0)])))
    return Workload(f"batched_{count}", cloths, 5, 10, frames, seed=seed)


def partition_cloths(costs, world: int) -> list[list[int]]:
    """Splits cloth indices over `world` GPUs, balancing the summed cost (particles x
    substeps x iterations): longest-processing-time-first greedy, ties to the lower
    rank.  Deterministic, so every rank computes the same partition without talking."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def shard(wl: Workload, rank: int, world: int) -> Workload:
    """The cloths of `wl` that rank `rank` of `world` simulates (strong scaling)."""
    costs = [c.num_particles * wl.substeps * wl.iterations for c in wl.cloths]
    mine = partition_cloths(costs, world)[rank]
    return Workload(f"{wl.name}_shard{rank}of{world}", [wl.cloths[i] for i in mine], wl.substeps,
                    wl.iterations, wl.frames, wl.relaxation, wl.friction, wl.collision_margin,
                    wl.frame_dt, wl.seed, dict(wl.notes, shard=(rank, world)))


def build_plain(spec: ClothSpec, solver, params_scalar: float = 1.5) -> int:
    """Registers one cloth the way VtClothObjectGPU::Start does (AddCloth, then
    GenerateStretch / GenerateAttach / GenerateBending); returns the offset."""
    verts, idx = spec.mesh()
    d = spec.particle_diameter(params_scalar)
    off = solver.add_cloth(verts, idx, spec.model, d)
    solver.build_grid_constraints(off, spec.resolution, spec.attached)
    solver.update_colliders(spec.colliders(0))
    return off
