"""GPU: the CUDA solver against what the reference's own solver kernels computed
(tests/golden/ref_*.npz, see tests/test_ref_pinning.py), bit for bit, through the C ABI —
the scenes of tests/ref_scenes.py (every collider kind, the schedule's branches, a whole
row of attachments, two cloths colliding) and HashObjects on a point cloud.  Needs neither
the oracle nor the reference on the GPU machine."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import ref_scenes
import velvet_gb300 as vg
from velvet_gb300 import _abi

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
EXACT = _abi.VARIANT != "fast"  # the fast build is held to a tolerance, not to bits


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def same(a, b, what):
    if not np.array_equal(bits(a), bits(b)):
        d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
        raise AssertionError(f"{what}: {(bits(a) != bits(b)).sum()} values differ, max |diff| {np.nanmax(d):.3g}")


@pytest.mark.skipif(not EXACT, reason="bit-exact comparison applies to the exact build")
@pytest.mark.parametrize("grid", [True, False], ids=["tile", "csr"])
@pytest.mark.parametrize("name", sorted(ref_scenes.SCENES))
def test_cuda_solver_reproduces_the_reference_kernels(name, grid):
    g = np.load(GOLDEN / f"{name}.npz")
    s = vg.ClothSolver(ref_scenes.params_for(name))
    if not grid:
        assert vg.lib().vt_solver_use_grid_kernel(s.handle, 0) == 0
    rec, normals = ref_scenes.run(name, s)
    for f, (x, v) in rec.items():
        same(x, g[f"positions_{f}"], f"{name}: positions after {f} frames")
        same(v, g[f"velocities_{f}"], f"{name}: velocities after {f} frames")
    same(normals, g["normals"], f"{name}: normals")
    if ref_scenes.SCENES[name]["params"].get("enable_self_collision", 1):
        for k, what in (("particle_hash", _abi.DEBUG_PARTICLE_HASH), ("particle_index", _abi.DEBUG_PARTICLE_INDEX),
                        ("cell_start", _abi.DEBUG_CELL_START)):
            assert np.array_equal(s.debug_view(what), g[k]), f"{name}: {k} of the last hash"
    s.close()


def test_hash_objects_reproduces_the_reference():
    torch = pytest.importorskip("torch")
    c = ref_scenes.HASH_CLOUD
    pos, orig = ref_scenes.hash_cloud_inputs()
    g = np.load(GOLDEN / "ref_hash_cloud.npz")
    n, T, mn = c["n"], c["table"], c["max_neighbors"]
    dev = torch.device("cuda")
    P, O = torch.from_numpy(pos.reshape(-1)).to(dev), torch.from_numpy(orig.reshape(-1)).to(dev)
    out = dict(hash=torch.empty(n, dtype=torch.int32, device=dev), index=torch.empty(n, dtype=torch.int32, device=dev),
               cell_start=torch.empty(T + 1, dtype=torch.int32, device=dev),
               cell_end=torch.zeros(T, dtype=torch.int32, device=dev),
               neighbors=torch.full((n * mn,), -1, dtype=torch.int32, device=dev))
    hp = _abi.VtHashParams(n, mn, c["spacing"], float(np.float32(c["spacing"]) * np.float32(c["spacing"])), T,
                           float(np.float32(c["diameter"]) * np.float32(c["diameter"])))
    _abi.check(vg.lib().vt_hash_objects(*(C.c_void_p(out[k].data_ptr()) for k in
                                          ("hash", "index", "cell_start", "cell_end", "neighbors")),
                                        C.c_void_p(P.data_ptr()), C.c_void_p(O.data_ptr()), C.byref(hp), None),
               "vt_hash_objects")
    torch.cuda.synchronize()
    r = {k: v.cpu().numpy().view(np.uint32) for k, v in out.items()}
    assert np.array_equal(r["hash"], g["particle_hash"])
    assert np.array_equal(r["index"], g["particle_index"])
    assert np.array_equal(r["cell_start"], g["cell_start"])
    occ = g["cell_start"][:-1] != 0xFFFFFFFF
    assert np.array_equal(r["cell_end"][occ], g["cell_end"][occ])

    def lists(nb):
        nb = nb.reshape(mn, n).astype(np.int64)
        end = nb == 0xFFFFFFFF
        return np.where((np.cumsum(end, axis=0) - end) > 0, -2, nb)

    assert np.array_equal(lists(r["neighbors"]), lists(g["neighbors"]))
