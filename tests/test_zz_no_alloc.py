"""GPU: the allocation-free spatial hash (vt_hash_objects_noalloc).

Callers that may not allocate device memory after start-up (fixed-budget engines, hosts
that own every allocation, real-time loops that cannot afford the device
synchronisation cudaMalloc implies) use this entry point; its sort scratch is a fixed
array compiled into the library.  These tests call it through the C ABI and check its
outputs against vt_hash_objects and the oracle's HashObjects on the same inputs, twice in
a row with different inputs (the shared scratch keeps the previous call's contents, which
must not matter), and once at the largest accepted table, VT_HASH_NOALLOC_MAX_OBJECTS
objects, around which the device's free memory must not change.  The hash is integer
work, so every comparison is exact.  This file is collected last so that a run stopping
at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import velvet_gb300 as vg
from velvet_gb300 import _abi

pytestmark = pytest.mark.gpu

MAX_OBJECTS = 262144  # VT_HASH_NOALLOC_MAX_OBJECTS


def _valid_lists(nb, n, mn):
    nb = nb.reshape(mn, n).astype(np.int64)
    end = nb == 0xFFFFFFFF
    after = (np.cumsum(end, axis=0) - end) > 0
    return np.where(after, -2, nb)


def _buffers(torch, n, mn):
    T = 2 * n
    dev = torch.device("cuda")
    return dict(hash=torch.empty(n, dtype=torch.int32, device=dev),
                index=torch.empty(n, dtype=torch.int32, device=dev),
                cell_start=torch.empty(T + 1, dtype=torch.int32, device=dev),
                cell_end=torch.zeros(T, dtype=torch.int32, device=dev),
                neighbors=torch.full((n * mn,), -1, dtype=torch.int32, device=dev))


def _call(fn, out, P, O, n, spacing, diam, mn):
    hp = _abi.VtHashParams(n, mn, spacing, float(np.float32(spacing) * np.float32(spacing)), 2 * n,
                           float(np.float32(diam) * np.float32(diam)))
    st = getattr(vg.lib(), fn)(*(C.c_void_p(out[k].data_ptr()) for k in
                                 ("hash", "index", "cell_start", "cell_end", "neighbors")),
                               C.c_void_p(P.data_ptr()), C.c_void_p(O.data_ptr()), C.byref(hp), None)
    _abi.check(st, fn)


def _run(torch, fn, pos, orig, spacing, diam, mn):
    n = pos.shape[0]
    P = torch.from_numpy(pos).cuda()
    O = torch.from_numpy(orig).cuda()
    out = _buffers(torch, n, mn)
    _call(fn, out, P, O, n, spacing, diam, mn)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy().view(np.uint32) for k, v in out.items()}


def _cloud(rng, n, half=0.25):
    pos = rng.uniform(-half, half, (n, 3)).astype(np.float32)
    pos[:, 1] *= 0.2  # a sheet-like cloud: dense cells, many neighbours
    orig = (pos + rng.normal(0.0, 0.02, (n, 3))).astype(np.float32)
    return pos, orig


def _assert_same_hash(a, b, n, mn, what):
    assert np.array_equal(a["hash"], b["hash"]), f"{what}: keys"
    assert np.array_equal(a["index"], b["index"]), f"{what}: sort order"
    assert np.array_equal(a["cell_start"], b["cell_start"]), f"{what}: cell_start"
    occ = a["cell_start"][:-1] != 0xFFFFFFFF  # cell_end is defined for occupied cells only
    assert np.array_equal(a["cell_end"][occ], b["cell_end"][occ]), f"{what}: cell_end"
    la, lb = _valid_lists(a["neighbors"], n, mn), _valid_lists(b["neighbors"], n, mn)
    assert np.array_equal(la, lb), f"{what}: neighbour lists"
    assert (la >= 0).sum() > n, "lists should not be empty"


def _oracle(pos, orig, spacing, diam, mn):
    o = oracle.hash_objects(pos, orig, spacing, 2 * pos.shape[0], mn, diam)
    return {"hash": o["particle_hash"], "index": o["particle_index"], "cell_start": o["cell_start"],
            "cell_end": o["cell_end"], "neighbors": o["neighbors"]}


def test_noalloc_hash_matches_allocating_hash_and_oracle_on_two_calls():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    spacing, diam, mn = 0.045, 0.03, 64
    for call, n in enumerate((5000, 12345)):
        pos, orig = _cloud(rng, n)
        a = _run(torch, "vt_hash_objects", pos, orig, spacing, diam, mn)
        b = _run(torch, "vt_hash_objects_noalloc", pos, orig, spacing, diam, mn)
        _assert_same_hash(a, b, n, mn, f"call {call}, no-alloc vs allocating")
        _assert_same_hash(_oracle(pos, orig, spacing, diam, mn), b, n, mn, f"call {call}, no-alloc vs oracle")


def test_noalloc_at_the_maximum_size_allocates_nothing():
    """VT_HASH_NOALLOC_MAX_OBJECTS objects (64 sort tiles, the whole scratch array): the
    same results as vt_hash_objects, and a warm call leaves the device's free memory
    unchanged."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(12)
    n, spacing, diam, mn = MAX_OBJECTS, 0.02, 0.012, 32
    pos, orig = _cloud(rng, n, half=0.8)  # about 2.6 objects per cell
    a = _run(torch, "vt_hash_objects", pos, orig, spacing, diam, mn)
    P, O = torch.from_numpy(pos).cuda(), torch.from_numpy(orig).cuda()
    out = _buffers(torch, n, mn)
    _call("vt_hash_objects_noalloc", out, P, O, n, spacing, diam, mn)  # first call: set-up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _call("vt_hash_objects_noalloc", out, P, O, n, spacing, diam, mn)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    b = {k: v.cpu().numpy().view(np.uint32) for k, v in out.items()}
    _assert_same_hash(a, b, n, mn, "maximum size")


def test_noalloc_rejects_oversize_tables():
    torch = pytest.importorskip("torch")
    cs = torch.empty(1, dtype=torch.int32, device="cuda")
    n = MAX_OBJECTS + 1  # refused on the host, nothing launched
    hp = _abi.VtHashParams(n, 64, 0.045, 0.045 * 0.045, 2 * n, 0.03 * 0.03)
    st = vg.lib().vt_hash_objects_noalloc(None, None, C.c_void_p(cs.data_ptr()), None, None, None, None,
                                          C.byref(hp), None)
    assert st == _abi.VT_ERR_CAPACITY
    assert b"262144" in vg.lib().vt_last_error()
