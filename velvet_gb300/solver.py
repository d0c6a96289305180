"""ClothSolver — Python face of the C ABI, shaped like VtClothSolverGPU.

Method names follow Velvet/VtClothSolverGPU.hpp:114-205 (AddCloth -> add_cloth, ...).
All arrays are numpy; vectors are (n, 3) float32, matrices 4x4 float32 in the usual
row/column math layout (converted to glm's column-major order at the boundary).
Every call goes through libvelvet_gb300.so; a failing status raises VtError.
"""
from __future__ import annotations

import ctypes as C
from typing import Iterable, Optional, Sequence

import numpy as np

from . import _abi
from ._abi import VtParams, VtSdfCollider, check, lib


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def colmajor(m: np.ndarray) -> np.ndarray:
    """4x4 (or 3x3) matrix -> flat column-major float32 (glm memory order)."""
    return np.ascontiguousarray(np.asarray(m, dtype=np.float32).T).reshape(-1)


def stream_handle(stream) -> C.c_void_p | None:
    """Accepts None, an int handle, or an object with .cuda_stream (torch.cuda.Stream)."""
    if stream is None:
        return None
    h = getattr(stream, "cuda_stream", stream)
    return C.c_void_p(int(h)) if h else None


def render_params(width: int, height: int, eye: Sequence[float], target: Sequence[float],
                  particle_radius: float, up: Sequence[float] = (0.0, 1.0, 0.0), fov_y_deg: float = 45.0,
                  z_near: float = 0.01, z_far: float = 100.0, light_dir: Sequence[float] = (0.3, 0.9, 0.3),
                  tint: Sequence[float] = (0.2, 0.3, 0.6), ambient: float = 0.3,
                  background: int = 0xFF262626) -> _abi.VtRenderParams:
    """vt_render_params for a perspective camera at `eye` looking at `target` (the
    matrices built by vt_camera_look_at / vt_camera_perspective)."""
    rp = _abi.VtRenderParams()
    rp.width, rp.height = width, height
    f3 = lambda v: (C.c_float * 3)(*[float(a) for a in v])  # noqa: E731
    check(lib().vt_camera_look_at(f3(eye), f3(target), f3(up), rp.view), "vt_camera_look_at")
    check(lib().vt_camera_perspective(float(np.radians(fov_y_deg)), width / height, z_near, z_far, rp.projection),
          "vt_camera_perspective")
    rp.z_near = z_near
    rp.particle_radius = particle_radius
    L = np.asarray(light_dir, np.float64)
    rp.light_dir[:] = [float(v) for v in (L / np.linalg.norm(L)).astype(np.float32)]
    rp.tint[:] = [float(v) for v in tint]
    rp.ambient = ambient
    rp.background = background
    return rp


def rgba_to_rgb(img: np.ndarray) -> np.ndarray:
    """(H, W) RGBA8 words (red in the low byte) -> (H, W, 3) uint8."""
    return np.ascontiguousarray(img, np.uint32).view(np.uint8).reshape(img.shape + (4,))[..., :3]


def write_ppm(path, img: np.ndarray) -> None:
    """Writes an RGBA8 image as binary PPM (P6)."""
    rgb = rgba_to_rgb(img)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (rgb.shape[1], rgb.shape[0]))
        f.write(rgb.tobytes())


# Variants of the grid tile kernel, by index (vt_tuning_set_grid_tile): (tile rows, tile
# columns, resident blocks per SM).
GRID_VARIANTS = ((7, 31, 4), (15, 15, 4), (3, 63, 4), (7, 31, 5), (15, 15, 5), (3, 63, 5))


def grid_variant_name(v: int) -> Optional[str]:
    """'15x15 x4/SM', or None for -1 (not chosen yet)."""
    if v < 0:
        return None
    ta, tb, blocks = GRID_VARIANTS[v]
    return f"{ta}x{tb} x{blocks}/SM"


class ClothSolver:
    """One plain solver domain (all its cloths share one hash and parameter block)."""

    def __init__(self, params: VtParams | None = None):
        self._h = C.c_void_p()
        p = params if params is not None else _abi.default_params()
        check(lib().vt_solver_create(C.byref(p), C.byref(self._h)), "vt_solver_create")

    # ------------------------------------------------------------------ lifetime
    def close(self) -> None:
        if self._h:
            lib().vt_solver_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # ------------------------------------------------------------------ params
    @property
    def params(self) -> VtParams:
        p = VtParams()
        check(lib().vt_solver_get_params(self._h, C.byref(p)), "vt_solver_get_params")
        return p

    @params.setter
    def params(self, p: VtParams) -> None:
        check(lib().vt_solver_set_params(self._h, C.byref(p)), "vt_solver_set_params")

    @property
    def num_particles(self) -> int:
        n = C.c_uint32()
        check(lib().vt_solver_num_particles(self._h, C.byref(n)), "vt_solver_num_particles")
        return n.value

    # ------------------------------------------------------------------ registration
    def add_cloth(self, vertices: np.ndarray, indices: np.ndarray, model: np.ndarray,
                  particle_diameter: float) -> int:
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        ind = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
        m = colmajor(model)
        off = C.c_int32()
        check(lib().vt_cloth_add(self._h, _ptr(v), v.shape[0], _ptr(ind), ind.size, _ptr(m),
                                 float(particle_diameter), C.byref(off)), "vt_cloth_add")
        return off.value

    def add_stretch(self, pairs: np.ndarray, rest: np.ndarray) -> None:
        pr = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        r = np.ascontiguousarray(rest, dtype=np.float32).reshape(-1)
        check(lib().vt_stretch_add(self._h, _ptr(pr), _ptr(r), r.size), "vt_stretch_add")

    def add_attach_slot(self, xyz: Sequence[float]) -> int:
        a = np.ascontiguousarray(xyz, dtype=np.float32).reshape(3)
        out = C.c_int32()
        check(lib().vt_attach_slot_add(self._h, _ptr(a), C.byref(out)), "vt_attach_slot_add")
        return out.value

    def add_attach(self, particles, slots, distances) -> None:
        p = np.ascontiguousarray(particles, dtype=np.int32).reshape(-1)
        s = np.ascontiguousarray(slots, dtype=np.int32).reshape(-1)
        d = np.ascontiguousarray(distances, dtype=np.float32).reshape(-1)
        check(lib().vt_attach_add(self._h, _ptr(p), _ptr(s), _ptr(d), p.size), "vt_attach_add")

    def generate_lra(self, first_slot: int, num_slots: int, particle_begin: int,
                     particle_count: int) -> None:
        check(lib().vt_attach_generate_lra(self._h, first_slot, num_slots, particle_begin,
                                           particle_count), "vt_attach_generate_lra")

    def add_bend(self, quads: np.ndarray, angles: np.ndarray) -> None:
        q = np.ascontiguousarray(quads, dtype=np.uint32).reshape(-1, 4)
        a = np.ascontiguousarray(angles, dtype=np.float32).reshape(-1)
        check(lib().vt_bend_add(self._h, _ptr(q), _ptr(a), a.size), "vt_bend_add")

    def build_grid_constraints(self, offset: int, resolution: int, attached: Iterable[int]) -> None:
        at = np.ascontiguousarray(list(attached), dtype=np.int32)
        check(lib().vt_cloth_build_grid_constraints(self._h, offset, resolution,
                                                    _ptr(at) if at.size else None, at.size),
              "vt_cloth_build_grid_constraints")

    def build_bending_adjacency(self, offset: int) -> int:
        """One bend per interior edge of the cloth at `offset`; returns how many."""
        n = C.c_uint32()
        check(lib().vt_cloth_build_bending_adjacency(self._h, offset, C.byref(n)),
              "vt_cloth_build_bending_adjacency")
        return n.value

    def update_colliders(self, colliders: Sequence[VtSdfCollider]) -> None:
        arr = (VtSdfCollider * max(1, len(colliders)))(*colliders)
        check(lib().vt_colliders_set(self._h, arr, len(colliders)), "vt_colliders_set")

    # ------------------------------------------------------------------ simulate
    def simulate(self, frame_dt: float, substeps: int, iterations: int, relaxation: float,
                 friction: float, collision_margin: float, particle_diameter: float,
                 stream=None) -> None:
        check(lib().vt_simulate(self._h, frame_dt, substeps, iterations, relaxation, friction,
                                collision_margin, particle_diameter, stream_handle(stream)),
              "vt_simulate")

    def sync(self) -> None:
        check(lib().vt_solver_sync(self._h), "vt_solver_sync")

    # ------------------------------------------------------------------ state
    def _get3(self, fn: str, first: int, count: int | None) -> np.ndarray:
        n = self.num_particles
        count = n - first if count is None else count
        out = np.empty((count, 3), dtype=np.float32)
        check(getattr(lib(), fn)(self._h, first, count, _ptr(out), 0, None), fn)
        return out

    def positions(self, first: int = 0, count: int | None = None) -> np.ndarray:
        return self._get3("vt_positions_get", first, count)

    def velocities(self, first: int = 0, count: int | None = None) -> np.ndarray:
        return self._get3("vt_velocities_get", first, count)

    def normals(self, first: int = 0, count: int | None = None) -> np.ndarray:
        return self._get3("vt_normals_get", first, count)

    def set_positions(self, xyz: np.ndarray, first: int = 0) -> None:
        a = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        check(lib().vt_positions_set(self._h, first, a.shape[0], _ptr(a), 0, None), "vt_positions_set")

    def set_velocities(self, xyz: np.ndarray, first: int = 0) -> None:
        a = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        check(lib().vt_velocities_set(self._h, first, a.shape[0], _ptr(a), 0, None), "vt_velocities_set")

    def inv_mass(self, first: int = 0, count: int | None = None) -> np.ndarray:
        n = self.num_particles
        count = n - first if count is None else count
        out = np.empty(count, dtype=np.float32)
        check(lib().vt_inv_mass_get(self._h, first, count, _ptr(out)), "vt_inv_mass_get")
        return out

    def set_inv_mass(self, w: np.ndarray, first: int = 0) -> None:
        a = np.ascontiguousarray(w, dtype=np.float32).reshape(-1)
        check(lib().vt_inv_mass_set(self._h, first, a.size, _ptr(a)), "vt_inv_mass_set")

    def set_attach_slot(self, slot: int, xyz: Sequence[float]) -> None:
        a = np.ascontiguousarray(xyz, dtype=np.float32).reshape(3)
        check(lib().vt_attach_slot_set(self._h, slot, _ptr(a)), "vt_attach_slot_set")

    def grid_tile(self) -> int:
        """Grid kernel variant in use (an index of GRID_VARIANTS; -1 before the first simulate)."""
        v = C.c_int32()
        check(lib().vt_solver_grid_tile(self._h, C.byref(v)), "vt_solver_grid_tile")
        return v.value

    def save_state(self) -> bytes:
        """Checkpoint (vt_solver_state_save): positions, velocities, inverse masses, slots."""
        n = C.c_uint64()
        check(lib().vt_solver_state_size(self._h, C.byref(n)), "vt_solver_state_size")
        buf = (C.c_char * n.value)()
        check(lib().vt_solver_state_save(self._h, buf, n.value), "vt_solver_state_save")
        return bytes(buf)

    def load_state(self, state: bytes) -> None:
        """Resume from save_state() of a solver registered the same way."""
        buf = C.create_string_buffer(state, len(state))
        check(lib().vt_solver_state_load(self._h, buf, len(state)), "vt_solver_state_load")

    def render(self, rp: _abi.VtRenderParams, stream=None) -> np.ndarray:
        """The particles as shaded spheres (vt_solver_render): (height, width) RGBA8."""
        out = np.empty((rp.height, rp.width), np.uint32)
        check(lib().vt_solver_render(self._h, C.byref(rp), _ptr(out), 0, stream_handle(stream)), "vt_solver_render")
        return out

    # ------------------------------------------------------------------ hash views
    def table_size(self) -> int:
        out = np.zeros(1, dtype=np.int32)
        check(lib().vt_solver_debug_get(self._h, _abi.DEBUG_TABLE_SIZE, _ptr(out), 4),
              "vt_solver_debug_get")
        return int(out[0])

    def debug_view(self, what: int) -> np.ndarray:
        n = self.num_particles
        T = self.table_size()
        mn = self.params.max_num_neighbors
        shape, dt = {
            _abi.DEBUG_PARTICLE_HASH: (n, np.uint32),
            _abi.DEBUG_PARTICLE_INDEX: (n, np.uint32),
            _abi.DEBUG_CELL_START: (T + 1, np.uint32),
            _abi.DEBUG_CELL_END: (T, np.uint32),
            _abi.DEBUG_NEIGHBORS: (n * mn, np.uint32),
            _abi.DEBUG_PREDICTED: ((n, 3), np.float32),
        }[what]
        out = np.empty(shape, dtype=dt)
        check(lib().vt_solver_debug_get(self._h, what, _ptr(out), out.nbytes), "vt_solver_debug_get")
        return out


class BatchSolver:
    """Many independent cloths advanced together (vt_batch_*).

    Each cloth is registered on its own ClothSolver and copied in with `add`; inside the
    batch it keeps its own hash, parameters, colliders and slots, so its result equals
    the same ClothSolver simulated alone.
    """

    def __init__(self):
        self._h = C.c_void_p()
        check(lib().vt_batch_create(C.byref(self._h)), "vt_batch_create")
        self.sizes: list[int] = []

    def close(self) -> None:
        if self._h:
            lib().vt_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def add(self, cloth: ClothSolver) -> int:
        idx = C.c_int32()
        check(lib().vt_batch_add(self._h, cloth.handle, C.byref(idx)), "vt_batch_add")
        self.sizes.append(cloth.num_particles)
        return idx.value

    @property
    def num_cloths(self) -> int:
        n = C.c_int32()
        check(lib().vt_batch_size(self._h, C.byref(n), None), "vt_batch_size")
        return n.value

    @property
    def num_particles(self) -> int:
        n = C.c_uint64()
        check(lib().vt_batch_size(self._h, None, C.byref(n)), "vt_batch_size")
        return n.value

    def update_colliders(self, index: int, colliders: Sequence[VtSdfCollider]) -> None:
        arr = (VtSdfCollider * max(1, len(colliders)))(*colliders)
        check(lib().vt_batch_colliders_set(self._h, index, arr, len(colliders)), "vt_batch_colliders_set")

    def set_attach_slot(self, index: int, slot: int, xyz: Sequence[float]) -> None:
        a = np.ascontiguousarray(xyz, dtype=np.float32).reshape(3)
        check(lib().vt_batch_attach_slot_set(self._h, index, slot, _ptr(a)), "vt_batch_attach_slot_set")

    def simulate(self, frame_dt: float, substeps: int, iterations: int, relaxation: float,
                 friction: float, collision_margin: float, particle_diameters=None, stream=None) -> None:
        d = None if particle_diameters is None else np.ascontiguousarray(particle_diameters, np.float32)
        check(lib().vt_batch_simulate(self._h, frame_dt, substeps, iterations, relaxation, friction,
                                      collision_margin, _ptr(d), stream_handle(stream)), "vt_batch_simulate")

    def sync(self) -> None:
        check(lib().vt_batch_sync(self._h), "vt_batch_sync")

    def _get(self, fn: str, index: int) -> np.ndarray:
        out = np.empty((self.sizes[index], 3), dtype=np.float32)
        check(getattr(lib(), fn)(self._h, index, _ptr(out), 0, None), fn)
        return out

    def positions(self, index: int) -> np.ndarray:
        return self._get("vt_batch_positions_get", index)

    def normals(self, index: int) -> np.ndarray:
        return self._get("vt_batch_normals_get", index)

    def velocities(self, index: int) -> np.ndarray:
        return self._get("vt_batch_velocities_get", index)

    def all_positions(self) -> np.ndarray:
        out = np.empty((sum(self.sizes), 3), dtype=np.float32)
        check(lib().vt_batch_all_get(self._h, 0, _ptr(out), 0, None), "vt_batch_all_get")
        return out

    def launch_count(self) -> int:
        v = C.c_uint64()
        check(lib().vt_batch_launch_count(self._h, C.byref(v)), "vt_batch_launch_count")
        return v.value

    def use_graphs(self, on: bool) -> None:
        check(lib().vt_batch_use_graphs(self._h, 1 if on else 0), "vt_batch_use_graphs")

    def grid_tile(self) -> int:
        """Grid kernel variant in use (an index of GRID_VARIANTS; -1 before the first simulate)."""
        v = C.c_int32()
        check(lib().vt_batch_grid_tile(self._h, C.byref(v)), "vt_batch_grid_tile")
        return v.value

    def render(self, rp: _abi.VtRenderParams, stream=None) -> np.ndarray:
        """Every cloth's particles as shaded spheres (vt_batch_render): (height, width) RGBA8."""
        out = np.empty((rp.height, rp.width), np.uint32)
        check(lib().vt_batch_render(self._h, C.byref(rp), _ptr(out), 0, stream_handle(stream)), "vt_batch_render")
        return out


class ClothServer:
    """Continuous batching of cloth requests (vt_server_*): submit grid cloths with a
    frame count, call tick() repeatedly; each tick retires, admits and advances every
    active request by one frame."""

    def __init__(self, hbm_budget_bytes: int, max_cloths: int = 1024, max_active_particles: int = 0,
                 frame_dt: float = 1 / 60, substeps: int = 5, iterations: int = 10, relaxation: float = 1.0,
                 friction: float = 0.1, collision_margin: float = 0.06):
        cfg = _abi.VtServerConfig(int(hbm_budget_bytes), max_cloths, max_active_particles, frame_dt, substeps,
                                  iterations, relaxation, friction, collision_margin)
        self.cfg = cfg
        self._h = C.c_void_p()
        check(lib().vt_server_create(C.byref(cfg), C.byref(self._h)), "vt_server_create")
        self.sizes: dict[int, int] = {}

    def close(self) -> None:
        if self._h:
            lib().vt_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, cloth: ClothSolver, frames: int) -> int:
        rid = C.c_int64()
        check(lib().vt_server_submit(self._h, cloth.handle, frames, C.byref(rid)), "vt_server_submit")
        self.sizes[rid.value] = cloth.num_particles
        return rid.value

    def submit_grid(self, resolution: int, cloth_size: float, model: np.ndarray, particle_diameter: float,
                    attached: Sequence[int], colliders: Sequence[VtSdfCollider], frames: int,
                    params: VtParams | None = None) -> int:
        """Queues a grid cloth by description (vt_server_submit_grid): the server builds
        its mesh, inverse masses and rest lengths on the device at admission."""
        g = _abi.VtGridCloth()
        g.resolution = resolution
        g.cloth_size = cloth_size
        g.model[:] = [float(v) for v in colmajor(model)]
        g.particle_diameter = particle_diameter
        at = (C.c_int32 * max(1, len(attached)))(*attached)
        g.attached = C.cast(at, C.POINTER(C.c_int32))
        g.n_attached = len(attached)
        cols = (VtSdfCollider * max(1, len(colliders)))(*colliders)
        rid = C.c_int64()
        check(lib().vt_server_submit_grid(self._h, C.byref(g), C.byref(params) if params is not None else None,
                                          cols, len(colliders), frames, C.byref(rid)), "vt_server_submit_grid")
        self.sizes[rid.value] = (resolution + 1) ** 2
        return rid.value

    def tick(self, stream=None) -> _abi.VtServerTickInfo:
        info = _abi.VtServerTickInfo()
        check(lib().vt_server_tick(self._h, stream_handle(stream), C.byref(info)), "vt_server_tick")
        return info

    def poll(self, rid: int) -> tuple[int, int]:
        st, done = C.c_int32(), C.c_int32()
        check(lib().vt_server_poll(self._h, rid, C.byref(st), C.byref(done)), "vt_server_poll")
        return st.value, done.value

    def cancel(self, rid: int) -> None:
        """vt_server_cancel: a queued request leaves at once, an active one at the next tick."""
        check(lib().vt_server_cancel(self._h, rid), "vt_server_cancel")

    def result(self, rid: int) -> np.ndarray:
        n = self.sizes[rid]
        out = np.empty((n, 3), np.float32)
        check(lib().vt_server_result(self._h, rid, _ptr(out), n), "vt_server_result")
        return out

    def stats(self) -> _abi.VtServerStats:
        s = _abi.VtServerStats()
        check(lib().vt_server_stats_get(self._h, C.byref(s)), "vt_server_stats_get")
        return s


def hash_objects(positions_dev: int, original_dev: int, n: int, cell_spacing: float,
                 table_size: int, max_neighbors: int, particle_diameter: float,
                 out_hash: int, out_index: int, out_cell_start: int, out_cell_end: int,
                 out_neighbors: int, stream=None) -> None:
    """HashObjects on device pointers (ints), see include/velvet_gb300.h."""
    hp = _abi.VtHashParams(n, max_neighbors, cell_spacing, np.float32(cell_spacing) * np.float32(cell_spacing),
                           table_size, np.float32(particle_diameter) * np.float32(particle_diameter))
    check(lib().vt_hash_objects(C.c_void_p(out_hash), C.c_void_p(out_index), C.c_void_p(out_cell_start),
                                C.c_void_p(out_cell_end), C.c_void_p(out_neighbors),
                                C.c_void_p(positions_dev), C.c_void_p(original_dev), C.byref(hp),
                                stream_handle(stream)), "vt_hash_objects")
