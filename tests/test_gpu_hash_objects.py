"""GPU parity of the exported spatial hash, vt_hash_objects (HashObjects,
Velvet/SpatialHashGPU.cu:159-196), against the oracle's restatement: cell keys, sort
order, cell ranges and neighbour lists of caller-owned float3 buffers are compared
exactly, on clouds dense enough to hit the per-cell and per-particle neighbour caps, on a
table with colliding buckets, and on empty and one-object inputs."""
import ctypes as C

import numpy as np
import pytest

import oracle
from velvet_gb300 import _abi
import velvet_gb300 as vg

pytestmark = pytest.mark.gpu


def _valid_lists(nb, n, mn):
    nb = nb.reshape(mn, n).astype(np.int64)
    end = nb == 0xFFFFFFFF
    after = (np.cumsum(end, axis=0) - end) > 0
    return np.where(after, -2, nb)


def _gpu(torch, pos, orig, spacing, T, mn, diam):
    n = pos.shape[0]
    dev = torch.device("cuda")
    P = torch.from_numpy(np.ascontiguousarray(pos, np.float32).reshape(-1)).to(dev)
    O = torch.from_numpy(np.ascontiguousarray(orig, np.float32).reshape(-1)).to(dev)
    out = dict(hash=torch.empty(max(n, 1), dtype=torch.int32, device=dev),
               index=torch.empty(max(n, 1), dtype=torch.int32, device=dev),
               cell_start=torch.empty(T + 1, dtype=torch.int32, device=dev),
               cell_end=torch.zeros(T, dtype=torch.int32, device=dev),
               neighbors=torch.full((max(n, 1) * mn,), -1, dtype=torch.int32, device=dev))
    hp = _abi.VtHashParams(n, mn, spacing, float(np.float32(spacing) * np.float32(spacing)), T,
                           float(np.float32(diam) * np.float32(diam)))
    _abi.check(vg.lib().vt_hash_objects(*(C.c_void_p(out[k].data_ptr()) for k in
                                          ("hash", "index", "cell_start", "cell_end", "neighbors")),
                                        C.c_void_p(P.data_ptr()), C.c_void_p(O.data_ptr()), C.byref(hp), None),
               "vt_hash_objects")
    torch.cuda.synchronize()
    r = {k: v.cpu().numpy().view(np.uint32) for k, v in out.items()}
    r["hash"], r["index"], r["neighbors"] = r["hash"][:n], r["index"][:n], r["neighbors"][:n * mn]
    return r


def _check(pos, orig, spacing, T, mn, diam):
    torch = pytest.importorskip("torch")
    n = pos.shape[0]
    g = _gpu(torch, pos, orig, spacing, T, mn, diam)
    o = oracle.hash_objects(pos, orig, spacing, T, mn, diam)
    assert np.array_equal(g["hash"], o["particle_hash"]), "keys"
    assert np.array_equal(g["index"], o["particle_index"]), "sort order"
    assert np.array_equal(g["cell_start"], o["cell_start"]), "cell_start"
    occ = o["cell_start"][:-1] != 0xFFFFFFFF
    assert np.array_equal(g["cell_end"][occ], o["cell_end"][occ]), "cell_end"
    if n:
        assert np.array_equal(_valid_lists(g["neighbors"], n, mn), _valid_lists(o["neighbors"], n, mn)), \
            "neighbour lists"
    return g


@pytest.mark.parametrize("n,half,mn", [(3000, 0.1, 64), (20000, 0.3, 64), (20000, 0.15, 8)])
def test_hash_objects_matches_the_oracle(n, half, mn):
    rng = np.random.default_rng(n + mn)
    pos = rng.uniform(-half, half, (n, 3)).astype(np.float32)
    pos[:, 1] *= 0.3
    orig = (pos + rng.normal(0.0, 0.03, (n, 3))).astype(np.float32)
    g = _check(pos, orig, 0.045, 2 * n, mn, 0.03)
    full = (_valid_lists(g["neighbors"], n, mn) >= 0).sum(axis=0) == mn
    if half <= 0.15:
        assert full.any(), "the dense cloud should fill some lists to the cap"


def test_hash_objects_small_table_collisions_and_negative_cells():
    """A table far smaller than the occupied cells (buckets shared by many cells) and
    coordinates on both sides of zero (floor of negative quotients, C remainder)."""
    rng = np.random.default_rng(5)
    n = 4000
    pos = rng.uniform(-2.0, 2.0, (n, 3)).astype(np.float32)
    orig = pos[rng.permutation(n)]
    _check(pos, orig, 0.05, 97, 64, 0.02)


def test_hash_objects_empty_and_single():
    _check(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32), 0.05, 16, 64, 0.03)
    one = np.array([[0.01, -0.02, 0.03]], np.float32)
    _check(one, one, 0.05, 2, 64, 0.03)


@pytest.mark.parametrize("n", [70_000, 4_000])
@pytest.mark.parametrize("T", [200, 40_000, 300_000, (1 << 25) + 1])
def test_hash_objects_sort_passes_one_to_four(T, n):
    """Tables whose key widths (8, 16, 19 and 26 bits) make the radix sort run one, two,
    three and four digit passes: an odd count starts from the temporaries, and every
    count must leave the sorted pairs in the caller's buffers.  70,000 objects span 18
    sort tiles, so each pass's look-back crosses tiles; 4,000 fit one tile, sorted by a
    single block with the pairs in shared memory between passes."""
    rng = np.random.default_rng(T + n)
    pos = rng.uniform(-1.0, 1.0, (n, 3)).astype(np.float32)
    pos[:, 1] *= 0.2
    orig = (pos + rng.normal(0.0, 0.05, (n, 3))).astype(np.float32)
    _check(pos, orig, 0.04, T, 32, 0.02)
