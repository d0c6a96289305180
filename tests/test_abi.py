"""CPU-only checks of the C ABI: the library loads, exports every function the public
header declares, and its host-side argument validation and parameter defaults behave
like the reference (no compute calls: there is no GPU here)."""
import ctypes as C
import re
from pathlib import Path

import pytest

import velvet_gb300 as vg
from velvet_gb300 import _abi

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> set[str]:
    text = (ROOT / "include" / "velvet_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return set(re.findall(r"\b(vt_[a-z0-9_]+)\s*\(", text))


def test_header_and_binding_agree():
    decl = declared_functions()
    assert decl, "no declarations parsed"
    assert decl == set(_abi.SIGNATURES), (decl ^ set(_abi.SIGNATURES))


def test_library_exports_every_declared_symbol():
    L = vg.lib()
    missing = [f for f in declared_functions() if not hasattr(L, f)]
    assert not missing, missing


def test_bounds_checked_build_exports_the_same_symbols():
    """build() also makes the bounds-checked library from the same sources."""
    path = Path(_abi.__file__).resolve().parent / "libvelvet_gb300_checked.so"
    assert path.exists(), "run __graft_entry__.build() first"
    L = C.CDLL(str(path))
    missing = [f for f in declared_functions() if not hasattr(L, f)]
    assert not missing, missing


def test_abi_version():
    assert vg.lib().vt_abi_version() == 1


def test_params_default_match_reference():
    # VtSimParams defaults, Velvet/Common.hpp:21-46
    p = vg.default_params()
    assert (p.num_substeps, p.num_iterations, p.max_num_neighbors) == (2, 4, 64)
    assert p.max_speed == 50.0
    assert list(p.gravity) == pytest.approx([0.0, -9.8, 0.0])
    assert p.bend_compliance == 0.0
    assert p.damping == 0.25 and p.relaxation_factor == 1.0
    assert p.long_range_stretchiness == pytest.approx(1.2)
    assert p.collision_margin == pytest.approx(0.06) and p.friction == pytest.approx(0.1)
    assert p.enable_self_collision == 1 and p.interleaved_hash == 3
    assert p.delta_time == pytest.approx(1 / 60)
    assert p.particle_diameter_scalar == 1.5 and p.hash_cell_size_scalar == 1.5


def test_params_struct_matches_oracle_defaults():
    import oracle

    a = vg.default_params()
    b = _abi.VtParams()
    oracle.lib().vo_params_default(C.byref(b))
    assert bytes(a) == bytes(b)


def test_status_strings():
    L = vg.lib()
    assert L.vt_status_string(0) == b"VT_OK"
    assert L.vt_status_string(-7) == b"VT_ERR_NUMERIC"


def test_host_validation_without_gpu():
    """Registration is host-side staging: it works and validates without a device."""
    import numpy as np

    s = vg.ClothSolver()
    verts = np.zeros((4, 3), np.float32)
    verts[:, 0] = [0, 1, 0, 1]
    verts[:, 1] = [0, 0, 1, 1]
    off = s.add_cloth(verts, [0, 1, 2, 2, 1, 3], np.eye(4), 1.5)
    assert off == 0 and s.num_particles == 4
    with pytest.raises(vg.VtError) as e:
        s.add_stretch([[0, 9]], [1.0])
    assert e.value.status == _abi.VT_ERR_INVALID_ARGUMENT
    with pytest.raises(vg.VtError):
        s.add_cloth(verts, [0, 1, 7], np.eye(4), 1.5)  # index out of range
    slot = s.add_attach_slot([0, 0, 0])
    s.add_attach([0], [slot], [0.0])  # distance 0 pins the particle
    assert s.inv_mass()[0] == 0.0
    s.set_inv_mass(np.array([0.5], np.float32), first=1)
    assert s.inv_mass()[1] == 0.5
    p = s.params
    assert p.particle_diameter == 1.5 and p.num_particles == 4
    # maxSpeed = 2 * d / fixedDt * substeps (VtClothSolverGPU.hpp:125)
    assert p.max_speed == pytest.approx(2 * 1.5 / (1 / 60) * 2, rel=1e-6)
    with pytest.raises(vg.VtError):
        s.simulate(1 / 60, 0, 1, 1, 0, 0, 1)  # zero substeps rejected before any launch
    s.close()
