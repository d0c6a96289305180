"""ctypes binding of the CPU oracle (oracle/libvt_oracle.so) — test infrastructure.

The oracle is a sequential C restatement of the reference GPU solver (see the header of
oracle/vt_oracle.c for the file:line map and its pinning status).  Tests use it as the
checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

from velvet_gb300._abi import VtHashParams, VtParams, VtSdfCollider

ROOT = Path(__file__).resolve().parents[1]
LIB = ROOT / "oracle" / "libvt_oracle.so"

GET_POSITIONS, GET_VELOCITIES, GET_PREDICTED, GET_NORMALS, GET_INV_MASS = 0, 1, 2, 3, 4
GET_HASH, GET_INDEX, GET_CELL_START, GET_CELL_END, GET_NEIGHBORS, GET_INITIAL = 5, 6, 7, 8, 9, 10

_L = None


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [ROOT / "oracle" / "vt_oracle.c", ROOT / "include" / "velvet_gb300.h"]
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def lib() -> C.CDLL:
    global _L
    if _L is None:
        if _stale():
            build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        sig = {
            "vo_params_default": (None, [C.POINTER(VtParams)]),
            "vo_create": (P, [C.POINTER(VtParams)]),
            "vo_destroy": (None, [P]),
            "vo_get_params": (None, [P, C.POINTER(VtParams)]),
            "vo_set_params": (None, [P, C.POINTER(VtParams)]),
            "vo_num_particles": (C.c_uint32, [P]),
            "vo_set_sum_order": (None, [P, C.c_int]),
            "vo_table_size": (C.c_int32, [P]),
            "vo_cloth_add": (C.c_int32, [P, P, C.c_uint32, P, C.c_uint32, P, C.c_float]),
            "vo_stretch_add": (None, [P, C.c_int32, C.c_int32, C.c_float]),
            "vo_attach_slot_add": (C.c_int32, [P, P]),
            "vo_attach_add": (None, [P, C.c_int32, C.c_int32, C.c_float]),
            "vo_bend_add": (None, [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float]),
            "vo_build_grid_constraints": (C.c_int, [P, C.c_int32, C.c_int32, P, C.c_uint32]),
            "vo_build_bending_adjacency": (C.c_int, [P, C.c_int32, C.POINTER(C.c_uint32)]),
            "vo_render": (None, [P, C.c_uint32, P, P]),
            "vo_colliders_set": (None, [P, P, C.c_uint32]),
            "vo_simulate": (None, [P, C.c_float, C.c_int32, C.c_int32, C.c_float, C.c_float,
                                   C.c_float, C.c_float]),
            "vo_get": (C.c_int, [P, C.c_int, P]),
            "vo_set_positions": (None, [P, C.c_uint32, C.c_uint32, P]),
            "vo_set_velocities": (None, [P, C.c_uint32, C.c_uint32, P]),
            "vo_set_inv_mass": (None, [P, C.c_uint32, C.c_uint32, P]),
            "vo_slot_set": (None, [P, C.c_int32, P]),
            "vo_num_constraints": (C.c_uint32, [P, C.c_int]),
            "vo_get_constraints": (None, [P, C.c_int, P, P]),
            "vo_acosf": (C.c_float, [C.c_float]),
            "vo_int_coord": (C.c_int32, [C.c_float, C.c_float]),
            "vo_hash_coords": (C.c_int32, [C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
            "vo_hash_objects": (None, [P, P, P, P, P, P, P, C.POINTER(VtHashParams)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _L = L
    return _L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


_CL = None
CPU_LIB = ROOT / "oracle" / "libvt_cpu_solver.so"


def cpu_solver_lib() -> C.CDLL:
    """oracle/libvt_cpu_solver.so: the reference's CPU solver restated (timing only)."""
    global _CL
    if _CL is None:
        src = ROOT / "oracle" / "vt_cpu_solver.c"
        if not CPU_LIB.exists() or src.stat().st_mtime > CPU_LIB.stat().st_mtime:
            build()
        L = C.CDLL(str(CPU_LIB))
        P = C.c_void_p
        L.vc_create.restype = P
        L.vc_create.argtypes = [P, C.c_int, P, C.c_int, P, C.c_int, P, C.c_int, C.POINTER(VtParams)]
        L.vc_destroy.argtypes = [P]
        L.vc_colliders_set.argtypes = [P, P, C.c_int]
        L.vc_simulate.argtypes = [P, C.c_float, C.c_int, C.c_int]
        L.vc_positions.argtypes = [P, P]
        _CL = L
    return _CL


class CpuSolver:
    """The reference's CPU solver (VtClothSolverCPU) on one grid cloth: timing only."""

    def __init__(self, spec, params: VtParams | None = None):
        p = params
        if p is None:
            p = VtParams()
            lib().vo_params_default(C.byref(p))
        verts, idx = spec.mesh()
        verts = np.ascontiguousarray(verts, np.float32)
        idx = np.ascontiguousarray(idx, np.uint32)
        m = colmajor(spec.model)
        at = np.ascontiguousarray(list(spec.attached), np.int32)
        self.n = verts.shape[0]
        self.h = cpu_solver_lib().vc_create(_p(verts), self.n, _p(idx), idx.size, _p(m), spec.resolution,
                                            _p(at) if at.size else None, at.size, C.byref(p))
        cols = spec.colliders(0)
        arr = (VtSdfCollider * max(1, len(cols)))(*cols)
        cpu_solver_lib().vc_colliders_set(self.h, arr, len(cols))

    def simulate(self, frame_dt, substeps, iterations):
        cpu_solver_lib().vc_simulate(self.h, frame_dt, substeps, iterations)

    def positions(self):
        out = np.empty((self.n, 3), np.float32)
        cpu_solver_lib().vc_positions(self.h, _p(out))
        return out

    def close(self):
        if self.h:
            cpu_solver_lib().vc_destroy(self.h)
            self.h = None


def colmajor(m) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(m, np.float32).T).reshape(-1)


class Oracle:
    """Sequential CPU solver with the same surface as velvet_gb300.ClothSolver."""

    def __init__(self, params: VtParams | None = None):
        p = params
        if p is None:
            p = VtParams()
            lib().vo_params_default(C.byref(p))
        self.h = lib().vo_create(C.byref(p))

    def close(self):
        if self.h:
            lib().vo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self) -> VtParams:
        p = VtParams()
        lib().vo_get_params(self.h, C.byref(p))
        return p

    @params.setter
    def params(self, p: VtParams):
        lib().vo_set_params(self.h, C.byref(p))

    @property
    def num_particles(self) -> int:
        return lib().vo_num_particles(self.h)

    def set_sum_order(self, reversed_: bool) -> None:
        """Reverse constraint order for the Jacobi sums: another valid order of the
        reference's unordered atomics."""
        lib().vo_set_sum_order(self.h, 1 if reversed_ else 0)

    def table_size(self) -> int:
        return lib().vo_table_size(self.h)

    def add_cloth(self, vertices, indices, model, diameter) -> int:
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        ind = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        m = colmajor(model)
        return lib().vo_cloth_add(self.h, _p(v), v.shape[0], _p(ind), ind.size, _p(m), float(diameter))

    def add_stretch(self, pairs, rest):
        pr = np.asarray(pairs, np.int32).reshape(-1, 2)
        r = np.asarray(rest, np.float32).reshape(-1)
        for (a, b), x in zip(pr, r):
            lib().vo_stretch_add(self.h, int(a), int(b), float(x))

    def add_attach_slot(self, xyz) -> int:
        a = np.ascontiguousarray(xyz, np.float32).reshape(3)
        return lib().vo_attach_slot_add(self.h, _p(a))

    def add_attach(self, particles, slots, distances):
        for p, s, d in zip(np.asarray(particles).reshape(-1), np.asarray(slots).reshape(-1),
                           np.asarray(distances, np.float32).reshape(-1)):
            lib().vo_attach_add(self.h, int(p), int(s), float(d))

    def add_bend(self, quads, angles):
        q = np.asarray(quads, np.uint32).reshape(-1, 4)
        for (a, b, c, d), x in zip(q, np.asarray(angles, np.float32).reshape(-1)):
            lib().vo_bend_add(self.h, int(a), int(b), int(c), int(d), float(x))

    def build_grid_constraints(self, offset, resolution, attached):
        at = np.ascontiguousarray(list(attached), np.int32)
        r = lib().vo_build_grid_constraints(self.h, offset, resolution, _p(at) if at.size else None, at.size)
        assert r == 0

    def build_bending_adjacency(self, offset):
        n = C.c_uint32()
        assert lib().vo_build_bending_adjacency(self.h, offset, C.byref(n)) == 0
        return n.value

    def update_colliders(self, cols):
        arr = (VtSdfCollider * max(1, len(cols)))(*cols)
        lib().vo_colliders_set(self.h, arr, len(cols))

    def simulate(self, frame_dt, substeps, iterations, relaxation, friction, margin, diameter):
        lib().vo_simulate(self.h, frame_dt, substeps, iterations, relaxation, friction, margin, diameter)

    def _get(self, what, shape, dt):
        out = np.empty(shape, dt)
        assert lib().vo_get(self.h, what, _p(out)) == 0
        return out

    def positions(self):
        return self._get(GET_POSITIONS, (self.num_particles, 3), np.float32)

    def velocities(self):
        return self._get(GET_VELOCITIES, (self.num_particles, 3), np.float32)

    def predicted(self):
        return self._get(GET_PREDICTED, (self.num_particles, 3), np.float32)

    def normals(self):
        return self._get(GET_NORMALS, (self.num_particles, 3), np.float32)

    def inv_mass(self):
        return self._get(GET_INV_MASS, (self.num_particles,), np.float32)

    def initial_positions(self):
        return self._get(GET_INITIAL, (self.num_particles, 3), np.float32)

    def hash_view(self):
        n, T, mn = self.num_particles, self.table_size(), self.params.max_num_neighbors
        return dict(
            particle_hash=self._get(GET_HASH, (n,), np.uint32),
            particle_index=self._get(GET_INDEX, (n,), np.uint32),
            cell_start=self._get(GET_CELL_START, (T + 1,), np.uint32),
            cell_end=self._get(GET_CELL_END, (T,), np.uint32),
            neighbors=self._get(GET_NEIGHBORS, (n * mn,), np.uint32),
        )

    def set_positions(self, xyz, first=0):
        a = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        lib().vo_set_positions(self.h, first, a.shape[0], _p(a))

    def set_velocities(self, xyz, first=0):
        a = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        lib().vo_set_velocities(self.h, first, a.shape[0], _p(a))

    def set_inv_mass(self, w, first=0):
        a = np.ascontiguousarray(w, np.float32).reshape(-1)
        lib().vo_set_inv_mass(self.h, first, a.size, _p(a))

    def set_attach_slot(self, slot, xyz):
        a = np.ascontiguousarray(xyz, np.float32).reshape(3)
        lib().vo_slot_set(self.h, slot, _p(a))

    def constraints(self, kind):
        n = lib().vo_num_constraints(self.h, kind)
        if kind == 0:
            ints, fl = np.empty(2 * n, np.int32), np.empty(n, np.float32)
        elif kind == 1:
            ints, fl = np.empty(2 * n, np.int32), np.empty(n, np.float32)
        else:
            ints, fl = np.empty(4 * n, np.int32), np.empty(n, np.float32)
        if n:
            lib().vo_get_constraints(self.h, kind, _p(ints), _p(fl))
        return ints, fl


def hash_objects(pos: np.ndarray, orig: np.ndarray, cell_spacing: float, table_size: int,
                 max_neighbors: int, diameter: float) -> dict:
    """HashObjects on host arrays (float3), reference layouts."""
    pos = np.ascontiguousarray(pos, np.float32)
    orig = np.ascontiguousarray(orig, np.float32)
    n = pos.shape[0]
    hp = VtHashParams(n, max_neighbors, cell_spacing, np.float32(cell_spacing) * np.float32(cell_spacing),
                      table_size, np.float32(diameter) * np.float32(diameter))
    out = dict(particle_hash=np.zeros(n, np.uint32), particle_index=np.zeros(n, np.uint32),
               cell_start=np.zeros(table_size + 1, np.uint32), cell_end=np.zeros(table_size, np.uint32),
               neighbors=np.zeros(n * max_neighbors, np.uint32))
    # the reference never clears cellEnd; give the oracle a T+1 buffer so its write at
    # index < T is all that matters
    ce = np.zeros(table_size + 1, np.uint32)
    lib().vo_hash_objects(_p(out["particle_hash"]), _p(out["particle_index"]), _p(out["cell_start"]),
                          _p(ce), _p(out["neighbors"]), _p(pos), _p(orig), C.byref(hp))
    out["cell_end"] = ce[:table_size]
    return out


def render(positions, rp):
    """The oracle's restatement of vt_solver_render on (n, 3) float32 positions."""
    x = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    out = np.empty((rp.height, rp.width), np.uint32)
    lib().vo_render(_p(x), x.shape[0], C.byref(rp), _p(out))
    return out
