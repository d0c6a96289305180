"""GPU: the allocation-free spatial hash (vt_hash_objects_noalloc).

Callers that may not allocate device memory after start-up (fixed-budget engines, hosts
that own every allocation, real-time loops that cannot afford the device
synchronisation cudaMalloc implies) use this entry point; its sort scratch is a fixed
array compiled into the library.  This test calls it through the C ABI and checks its
outputs against vt_hash_objects on the same inputs, twice in a row with different
inputs (the shared scratch keeps the previous call's contents, which must not matter).
The hash is integer work, so the comparison is exact.  This file is collected last so
that a run stopping at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

import velvet_gb300 as vg
from velvet_gb300 import _abi

pytestmark = pytest.mark.gpu


def _valid_lists(nb, n, mn):
    nb = nb.reshape(mn, n).astype(np.int64)
    end = nb == 0xFFFFFFFF
    after = (np.cumsum(end, axis=0) - end) > 0
    return np.where(after, -2, nb)


def _run(torch, fn, pos, orig, spacing, diam, mn):
    n = pos.shape[0]
    T = 2 * n
    dev = torch.device("cuda")
    P = torch.from_numpy(pos).to(dev)
    O = torch.from_numpy(orig).to(dev)
    out = dict(hash=torch.empty(n, dtype=torch.int32, device=dev),
               index=torch.empty(n, dtype=torch.int32, device=dev),
               cell_start=torch.empty(T + 1, dtype=torch.int32, device=dev),
               cell_end=torch.zeros(T, dtype=torch.int32, device=dev),
               neighbors=torch.full((n * mn,), -1, dtype=torch.int32, device=dev))
    hp = _abi.VtHashParams(n, mn, spacing, float(np.float32(spacing) * np.float32(spacing)), T,
                           float(np.float32(diam) * np.float32(diam)))
    st = getattr(vg.lib(), fn)(*(C.c_void_p(out[k].data_ptr()) for k in
                                 ("hash", "index", "cell_start", "cell_end", "neighbors")),
                               C.c_void_p(P.data_ptr()), C.c_void_p(O.data_ptr()), C.byref(hp), None)
    _abi.check(st, fn)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy().view(np.uint32) for k, v in out.items()}


def test_noalloc_hash_matches_allocating_hash_on_two_calls():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    spacing, diam, mn = 0.045, 0.03, 64
    for call, n in enumerate((5000, 12345)):
        pos = rng.uniform(-0.25, 0.25, (n, 3)).astype(np.float32)
        pos[:, 1] *= 0.2  # a sheet-like cloud: dense cells, many neighbours
        orig = (pos + rng.normal(0.0, 0.02, (n, 3))).astype(np.float32)
        a = _run(torch, "vt_hash_objects", pos, orig, spacing, diam, mn)
        b = _run(torch, "vt_hash_objects_noalloc", pos, orig, spacing, diam, mn)
        assert np.array_equal(a["hash"], b["hash"]), f"call {call}: keys"
        assert np.array_equal(a["index"], b["index"]), f"call {call}: sort order"
        assert np.array_equal(a["cell_start"], b["cell_start"]), f"call {call}: cell_start"
        occ = a["cell_start"][:-1] != 0xFFFFFFFF
        assert np.array_equal(a["cell_end"][occ], b["cell_end"][occ]), f"call {call}: cell_end"
        la, lb = _valid_lists(a["neighbors"], n, mn), _valid_lists(b["neighbors"], n, mn)
        assert np.array_equal(la, lb), f"call {call}: neighbour lists"
        assert (la >= 0).sum() > n, "lists should not be empty"


def test_noalloc_rejects_oversize_tables():
    torch = pytest.importorskip("torch")
    cs = torch.empty(1, dtype=torch.int32, device="cuda")
    n = 262144 + 1  # VT_HASH_NOALLOC_MAX_OBJECTS + 1: refused on the host, nothing launched
    hp = _abi.VtHashParams(n, 64, 0.045, 0.045 * 0.045, 2 * n, 0.03 * 0.03)
    st = vg.lib().vt_hash_objects_noalloc(None, None, C.c_void_p(cs.data_ptr()), None, None, None, None,
                                          C.byref(hp), None)
    assert st == _abi.VT_ERR_CAPACITY
    assert b"262144" in vg.lib().vt_last_error()
