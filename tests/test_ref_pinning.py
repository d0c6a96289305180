"""The oracle pinned to the reference's own code.

tests/golden/ref_*.npz hold what the reference's solver kernels (Velvet/VtClothSolverGPU.cu,
Velvet/SpatialHashGPU.cu, compiled unmodified for the CPU, see oracle/refemu) computed on the
scenes of tests/ref_scenes.py; the oracle must reproduce every recorded position, velocity,
normal, hash key, sorted index and cell start bit for bit, and the HashObjects output of a
point cloud (keys, order, cell ranges, neighbour lists).  Where the reference tree is present
the same comparison also runs live on the small configuration's full 64x64 cloth, and the
parameter defaults are read from the reference's Velvet/Common.hpp."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import oracle
import ref_scenes
import refemu
from oracle import Oracle
from velvet_gb300 import _abi
from velvet_gb300 import workloads as W

GOLDEN = Path(__file__).resolve().parent / "golden"


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same(a, b, what):
    if not np.array_equal(bits(a), bits(b)):
        d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
        raise AssertionError(f"{what}: {(bits(a) != bits(b)).sum()} values differ, max |diff| {np.nanmax(d):.3g}")


def valid_lists(nb, n, mn):
    nb = np.asarray(nb).reshape(mn, n).astype(np.int64)
    end = nb == 0xFFFFFFFF
    return np.where((np.cumsum(end, axis=0) - end) > 0, -2, nb)


@pytest.mark.parametrize("name", sorted(ref_scenes.SCENES))
def test_oracle_reproduces_the_reference_kernels(name):
    g = np.load(GOLDEN / f"{name}.npz")
    o = Oracle(ref_scenes.params_for(name))
    rec, normals = ref_scenes.run(name, o)
    for f, (x, v) in rec.items():
        same(x, g[f"positions_{f}"], f"{name}: positions after {f} frames")
        same(v, g[f"velocities_{f}"], f"{name}: velocities after {f} frames")
    same(normals, g["normals"], f"{name}: normals")
    if ref_scenes.SCENES[name]["params"].get("enable_self_collision", 1):
        hv = o.hash_view()
        for k in ("particle_hash", "particle_index", "cell_start"):
            assert np.array_equal(hv[k], g[k]), f"{name}: {k} of the last hash"


def test_scenes_move_and_collide():
    """The recorded scenes are not trivial: cloths fall, and the stress-shaped one is held
    by its attachments."""
    g = np.load(GOLDEN / "ref_stress24.npz")
    x0 = Oracle(ref_scenes.params_for("ref_stress24"))
    ref_scenes.register(x0, ref_scenes.specs("ref_stress24"))
    moved = np.abs(g["positions_16"] - x0.positions()).max()
    assert moved > 0.05
    g2 = np.load(GOLDEN / "ref_two_cloths.npz")
    assert g2["positions_24"].shape[0] == 16 * 16 + 12 * 12
    free = g2["positions_24"][256:]
    assert free[:, 1].max() < 0.3, "the free cloth should have fallen onto the pinned one"


def test_oracle_hash_objects_reproduces_the_reference():
    c = ref_scenes.HASH_CLOUD
    pos, orig = ref_scenes.hash_cloud_inputs()
    g = np.load(GOLDEN / "ref_hash_cloud.npz")
    o = oracle.hash_objects(pos, orig, c["spacing"], c["table"], c["max_neighbors"], c["diameter"])
    assert np.array_equal(o["particle_hash"], g["particle_hash"])
    assert np.array_equal(o["particle_index"], g["particle_index"])
    assert np.array_equal(o["cell_start"], g["cell_start"])
    occ = g["cell_start"][:-1] != 0xFFFFFFFF
    assert np.array_equal(o["cell_end"][occ], g["cell_end"][occ])
    n, mn = c["n"], c["max_neighbors"]
    ref_lists = valid_lists(g["neighbors"], n, mn)
    assert np.array_equal(valid_lists(o["neighbors"], n, mn), ref_lists)
    assert (ref_lists >= 0).sum(axis=0).max() == mn, "the cloud should fill some lists to the cap"


needs_ref = pytest.mark.skipif(not refemu.available(), reason="the reference tree is not on this machine")


@needs_ref
def test_oracle_equals_reference_kernels_live_on_the_small_configuration():
    """64x64, sphere + plane, 5 x 10, self-collision: 30 frames, every frame compared."""
    wl = W.small(frames=30)
    spec = wl.cloths[0]
    o, r = Oracle(), refemu.RefSolver()
    for s in (o, r):
        W.build_plain(spec, s)
    d = spec.particle_diameter()
    for f in range(wl.frames):
        for s in (o, r):
            s.simulate(wl.frame_dt, wl.substeps, wl.iterations, wl.relaxation, wl.friction,
                       wl.collision_margin, d)
        same(o.positions(), r.positions(), f"positions frame {f}")
        same(o.velocities(), r.velocities(), f"velocities frame {f}")
    same(o.normals(), r.normals(), "normals")
    ho, hr = o.hash_view(), r.hash_view()
    n, mn = o.num_particles, 64
    assert np.array_equal(valid_lists(ho["neighbors"], n, mn), valid_lists(hr["neighbors"], n, mn))


@needs_ref
def test_parameter_defaults_match_the_reference_header():
    """vt_params / the oracle's defaults against the HOST_INIT values of VtSimParams in the
    reference's Velvet/Common.hpp, read as text."""
    text = (refemu.REF_TREE / "Common.hpp").read_text(errors="replace")
    body = text[text.index("struct VtSimParams"):text.index("void OnGUI")]
    found = dict(re.findall(r"\b(\w+)\s+HOST_INIT\((.*?)\);", body))
    p = _abi.VtParams()
    oracle.lib().vo_params_default(C.byref(p))
    g = _abi.default_params() if hasattr(_abi, "default_params") else None
    names = {"numSubsteps": "num_substeps", "numIterations": "num_iterations",
             "maxNumNeighbors": "max_num_neighbors", "maxSpeed": "max_speed",
             "bendCompliance": "bend_compliance", "damping": "damping", "relaxationFactor": "relaxation_factor",
             "longRangeStretchiness": "long_range_stretchiness", "collisionMargin": "collision_margin",
             "friction": "friction", "enableSelfCollision": "enable_self_collision",
             "interleavedHash": "interleaved_hash", "particleDiameterScalar": "particle_diameter_scalar",
             "hashCellSizeScalar": "hash_cell_size_scalar"}
    assert set(names) <= set(found), sorted(set(names) - set(found))
    for ref_name, ours in names.items():
        raw = found[ref_name].strip().rstrip("f")
        want = 1.0 if raw == "true" else 0.0 if raw == "false" else float(raw)
        for src, params in (("oracle", p), ("library", g)):
            if params is not None:
                assert float(np.float32(getattr(params, ours))) == float(np.float32(want)), (src, ref_name)
    grav = [float(v.rstrip("f")) for v in re.findall(r"[-\d.]+f?", found["gravity"].split("(", 1)[1])]
    assert [float(v) for v in p.gravity] == [float(np.float32(v)) for v in grav]
