"""ctypes binding of oracle/_ref/libvr_ref.so — the reference's own solver kernels
(Velvet/VtClothSolverGPU.cu, Velvet/SpatialHashGPU.cu, compiled unmodified for the CPU
by `make -C oracle ref`, see oracle/refemu/vr_driver.cpp).  Test infrastructure: it pins
the oracle to the reference's code.  The library can only be built where the reference
tree exists; `available()` is False elsewhere and the tests that need it skip, while the
fixtures it produced (tests/golden/ref_*.npz, made by tests/golden/make_ref_golden.py)
travel with the repository."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from velvet_gb300._abi import VtHashParams, VtParams, VtSdfCollider

ROOT = Path(__file__).resolve().parents[1]
LIB = ROOT / "oracle" / "_ref" / "libvr_ref.so"
REF_TREE = Path(os.environ.get("VT_REFERENCE_TREE", "/root/reference/Velvet"))

_L = None


def available() -> bool:
    """True if the reference-kernel library exists or can be built here."""
    if LIB.exists():
        return True
    if not (REF_TREE / "VtClothSolverGPU.cu").exists():
        return False
    r = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref", f"REF={REF_TREE}"],
                       capture_output=True, text=True)
    return r.returncode == 0 and LIB.exists()


def lib() -> C.CDLL:
    global _L
    if _L is None:
        if not available():
            raise RuntimeError("oracle/_ref/libvr_ref.so is absent and the reference tree is not here")
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        sig = {
            "vr_create": (P, [C.POINTER(VtParams)]),
            "vr_destroy": (None, [P]),
            "vr_num_particles": (C.c_uint32, [P]),
            "vr_table_size": (C.c_int32, [P]),
            "vr_cloth_add": (C.c_int32, [P, P, C.c_uint32, P, C.c_uint32, P, C.c_float]),
            "vr_build_grid_constraints": (C.c_int, [P, C.c_int32, C.c_int32, P, C.c_uint32]),
            "vr_colliders_set": (None, [P, P, C.c_uint32]),
            "vr_simulate": (None, [P, C.c_float, C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_float,
                                   C.c_float]),
            "vr_get": (C.c_int, [P, C.c_int, P]),
            "vr_set_positions": (None, [P, C.c_uint32, C.c_uint32, P]),
            "vr_set_velocities": (None, [P, C.c_uint32, C.c_uint32, P]),
            "vr_hash_objects": (None, [P, P, P, P, P, P, P, C.POINTER(VtHashParams)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _L = L
    return _L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


class RefSolver:
    """The reference's kernels behind the surface of tests/oracle.Oracle."""

    def __init__(self, params: VtParams | None = None):
        import oracle

        p = params
        if p is None:
            p = VtParams()
            oracle.lib().vo_params_default(C.byref(p))
        self.max_neighbors = p.max_num_neighbors
        self.h = lib().vr_create(C.byref(p))

    def close(self):
        if self.h:
            lib().vr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_particles(self) -> int:
        return lib().vr_num_particles(self.h)

    def table_size(self) -> int:
        return lib().vr_table_size(self.h)

    def add_cloth(self, vertices, indices, model, diameter) -> int:
        v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        ind = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        m = np.ascontiguousarray(np.asarray(model, np.float32).T).reshape(-1)
        return lib().vr_cloth_add(self.h, _p(v), v.shape[0], _p(ind), ind.size, _p(m), float(diameter))

    def build_grid_constraints(self, offset, resolution, attached):
        at = np.ascontiguousarray(list(attached), np.int32)
        assert lib().vr_build_grid_constraints(self.h, offset, resolution, _p(at) if at.size else None,
                                               at.size) == 0

    def update_colliders(self, cols):
        arr = (VtSdfCollider * max(1, len(cols)))(*cols)
        lib().vr_colliders_set(self.h, arr, len(cols))

    def simulate(self, frame_dt, substeps, iterations, relaxation, friction, margin, diameter):
        lib().vr_simulate(self.h, frame_dt, substeps, iterations, relaxation, friction, margin, diameter)

    def _get(self, what, shape, dt):
        out = np.empty(shape, dt)
        assert lib().vr_get(self.h, what, _p(out)) == 0
        return out

    def positions(self):
        return self._get(0, (self.num_particles, 3), np.float32)

    def velocities(self):
        return self._get(1, (self.num_particles, 3), np.float32)

    def predicted(self):
        return self._get(2, (self.num_particles, 3), np.float32)

    def normals(self):
        return self._get(3, (self.num_particles, 3), np.float32)

    def inv_mass(self):
        return self._get(4, (self.num_particles,), np.float32)

    def hash_view(self):
        n, T = self.num_particles, self.table_size()
        return dict(particle_hash=self._get(5, (n,), np.uint32), particle_index=self._get(6, (n,), np.uint32),
                    cell_start=self._get(7, (T + 1,), np.uint32), cell_end=self._get(8, (T,), np.uint32),
                    neighbors=self._get(9, (n * self.max_neighbors,), np.uint32))

    def set_positions(self, xyz):
        a = np.ascontiguousarray(xyz, np.float32)
        lib().vr_set_positions(self.h, 0, a.shape[0], _p(a))

    def set_velocities(self, xyz):
        a = np.ascontiguousarray(xyz, np.float32)
        lib().vr_set_velocities(self.h, 0, a.shape[0], _p(a))


def hash_objects(pos, orig, cell_spacing, table_size, max_neighbors, diameter) -> dict:
    """The reference's HashObjects on host float3 arrays (cellStart with T + 1 entries)."""
    pos = np.ascontiguousarray(pos, np.float32)
    orig = np.ascontiguousarray(orig, np.float32)
    n = pos.shape[0]
    hp = VtHashParams(n, max_neighbors, cell_spacing, np.float32(cell_spacing) * np.float32(cell_spacing),
                      table_size, np.float32(diameter) * np.float32(diameter))
    out = dict(particle_hash=np.zeros(max(n, 1), np.uint32), particle_index=np.zeros(max(n, 1), np.uint32),
               cell_start=np.zeros(table_size + 1, np.uint32), cell_end=np.zeros(table_size + 1, np.uint32),
               neighbors=np.zeros(max(n, 1) * max_neighbors, np.uint32))
    lib().vr_hash_objects(_p(out["particle_hash"]), _p(out["particle_index"]), _p(out["cell_start"]),
                          _p(out["cell_end"]), _p(out["neighbors"]), _p(pos), _p(orig), C.byref(hp))
    out["particle_hash"], out["particle_index"] = out["particle_hash"][:n], out["particle_index"][:n]
    out["cell_end"], out["neighbors"] = out["cell_end"][:table_size], out["neighbors"][:n * max_neighbors]
    return out
