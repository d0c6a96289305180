"""GPU: the served form.  Requests of different sizes arrive while others are on the
GPU; each is admitted when a slot and memory free up, shares launches with the others,
and must end with exactly the bits it gets when simulated alone on the plain solver."""
import numpy as np
import pytest

import velvet_gb300 as vg
from velvet_gb300 import _abi
from velvet_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def request(side, height=0.6, mover=False):
    cols = W.moving_sphere(0.2, 0.2, 1.0) if mover else W.static_colliders([W.sphere((0, 0.3, 0), 0.3), W.plane(0)])
    return W.ClothSpec(side, 0.02, W.horizontal_cloth(side, 0.02, height), [0, side - 1], cols)


def alone(spec, frames, S=3, It=4):
    s = vg.ClothSolver()
    W.build_plain(spec, s)
    for _ in range(frames):
        s.simulate(float(W.FRAME_DT), S, It, 1.0, 0.1, 0.06, spec.particle_diameter())
    s.sync()
    return s.positions()


def registered(spec):
    s = vg.ClothSolver()
    W.build_plain(spec, s)
    return s


def test_staggered_requests_equal_alone():
    srv = vg.ClothServer(hbm_budget_bytes=2 << 30, max_cloths=8, substeps=3, iterations=4)
    plan = [(0, 20, 7), (0, 33, 12), (2, 9, 5), (3, 40, 9), (6, 16, 3)]  # (arrival tick, side, frames)
    ids, specs = {}, {}
    tick = 0
    while tick < 60:
        for t, side, frames in plan:
            if t == tick:
                spec = request(side, 0.5 + 0.01 * side)
                s = registered(spec)
                rid = srv.submit(s, frames)
                s.close()  # the server keeps its own copy
                ids[rid] = (side, frames)
                specs[rid] = spec
        info = srv.tick()
        tick += 1
        if tick > max(p[0] for p in plan) and info.active == 0 and info.queued == 0:
            break
    for rid, (side, frames) in ids.items():
        st, done = srv.poll(rid)
        assert st == _abi.REQ_DONE and done == frames
        got = srv.result(rid)
        want = alone(specs[rid], frames)
        assert np.array_equal(bits(got), bits(want)), f"request side {side}"
    stats = srv.stats()
    assert stats.requests_done == len(plan)
    assert stats.p99_frame_ms >= stats.p50_frame_ms > 0


def test_admission_waits_for_budget_and_cap():
    # a cap of 1000 active particles: the 32x32 request (1024) must wait until it runs alone
    srv = vg.ClothServer(hbm_budget_bytes=1 << 30, max_cloths=4, max_active_particles=1000,
                         substeps=2, iterations=2)
    a = registered(request(20))   # 400 particles
    b = registered(request(32))   # 1024 particles
    ra = srv.submit(a, 3)
    rb = srv.submit(b, 2)
    info = srv.tick()
    assert info.active == 1 and info.queued == 1
    assert srv.poll(rb)[0] == _abi.REQ_QUEUED
    for _ in range(40):
        srv.tick()
        (sa, da), (sb, db) = srv.poll(ra), srv.poll(rb)
        assert db == 0 or da == 3, "the large request ran beside the small one"
        if sa == _abi.REQ_DONE and sb == _abi.REQ_DONE:
            break
    assert srv.poll(ra) == (_abi.REQ_DONE, 3) and srv.poll(rb) == (_abi.REQ_DONE, 2)
    assert np.array_equal(bits(srv.result(rb)), bits(alone(request(32), 2, 2, 2)))
    assert np.array_equal(bits(srv.result(ra)), bits(alone(request(20), 3, 2, 2)))


def test_ticks_overlap_host_work_with_the_previous_frame():
    """A tick returns with its own frame still queued (it waits only for the previous
    one), so a result appears a tick or two after its last frame; ranges freed by
    finishing requests are reused at once.  Every request still ends with its bits
    when simulated alone."""
    srv = vg.ClothServer(hbm_budget_bytes=1 << 30, max_cloths=16, substeps=2, iterations=3)
    specs, ids = {}, []
    for k, side in enumerate([12, 40, 17, 64, 23, 9, 31, 50]):
        spec = request(side, 0.4 + 0.01 * k)
        s = registered(spec)
        rid = srv.submit(s, 2 + k % 3)
        s.close()
        specs[rid] = (spec, 2 + k % 3)
        ids.append(rid)
    for _ in range(60):
        info = srv.tick()
        if info.active == 0 and info.queued == 0:
            break
    for rid in ids:
        spec, frames = specs[rid]
        assert srv.poll(rid) == (_abi.REQ_DONE, frames)
        assert np.array_equal(bits(srv.result(rid)), bits(alone(spec, frames, 2, 3)))


def submit_described(srv, spec, frames):
    return srv.submit_grid(spec.resolution, spec.spacing * spec.resolution, spec.model, spec.particle_diameter(),
                           spec.attached, spec.colliders(0), frames)


def test_described_grid_cloths_built_on_the_device_equal_registered_ones():
    """vt_server_submit_grid builds mesh, inverse masses and rest lengths with a kernel at
    admission; mixed with host-registered requests, every result has the bits of the same
    cloth registered on the host and simulated alone."""
    srv = vg.ClothServer(hbm_budget_bytes=1 << 30, max_cloths=8, substeps=3, iterations=4)
    plan = [(request(20, 0.5), 5, True), (request(33, 0.53), 4, False), (request(9, 0.55), 6, True),
            (W.ClothSpec(17, 0.02, W.horizontal_cloth(17, 0.02, 0.45), [0, 8, 16, 280],
                         request(17).colliders), 3, True)]
    ids = []
    for spec, frames, described in plan:
        if described:
            rid = submit_described(srv, spec, frames)
        else:
            s = registered(spec)
            rid = srv.submit(s, frames)
            s.close()
        ids.append((rid, spec, frames))
    for _ in range(60):
        info = srv.tick()
        if info.active == 0 and info.queued == 0:
            break
    for rid, spec, frames in ids:
        assert srv.poll(rid) == (_abi.REQ_DONE, frames)
        assert np.array_equal(bits(srv.result(rid)), bits(alone(spec, frames))), f"side {spec.side}"


def test_described_grid_cloth_arguments_are_checked():
    srv = vg.ClothServer(hbm_budget_bytes=1 << 27, max_cloths=2)
    spec = request(12)
    with pytest.raises(vg.VtError) as e:
        srv.submit_grid(11, 0.22, spec.model, spec.particle_diameter(), [0, 1, 2, 3, 4], spec.colliders(0), 1)
    assert e.value.status == _abi.VT_ERR_CAPACITY  # more than four attach slots
    with pytest.raises(vg.VtError) as e:
        srv.submit_grid(11, 0.22, spec.model, spec.particle_diameter(), [144], spec.colliders(0), 1)
    assert e.value.status == _abi.VT_ERR_INVALID_ARGUMENT  # vertex out of range
    with pytest.raises(vg.VtError) as e:
        srv.submit_grid(699, 13.98, spec.model, spec.particle_diameter(), [0], spec.colliders(0), 1)
    assert e.value.status == _abi.VT_ERR_CAPACITY  # larger than the arena


def test_a_request_that_turns_nan_is_evicted_and_the_others_are_untouched():
    """Failure isolation: a request seeded with a NaN velocity raises its slot's fault flag
    in its first frame; the server evicts it (VT_REQ_FAILED, no result) and every other
    request of the mix still ends with its bits when simulated alone."""
    srv = vg.ClothServer(hbm_budget_bytes=1 << 30, max_cloths=8, substeps=3, iterations=4)
    good = [(request(20, 0.5), 6), (request(27, 0.55), 5)]
    ids = []
    for k, (spec, frames) in enumerate(good):
        s = registered(spec)
        ids.append((srv.submit(s, frames), spec, frames))
        s.close()
        if k == 0:  # the faulty one arrives between the two good ones
            bad = registered(request(16, 0.45))
            v = bad.velocities()
            v[7] = np.nan
            bad.set_velocities(v)
            bad_id = srv.submit(bad, 8)
            bad.close()
    for _ in range(60):
        info = srv.tick()
        if info.active == 0 and info.queued == 0:
            break
    st, done = srv.poll(bad_id)
    assert st == _abi.REQ_FAILED and done < 8
    with pytest.raises(vg.VtError) as e:
        srv.result(bad_id)
    assert e.value.status == _abi.VT_ERR_NUMERIC
    for rid, spec, frames in ids:
        assert srv.poll(rid) == (_abi.REQ_DONE, frames)
        assert np.array_equal(bits(srv.result(rid)), bits(alone(spec, frames)))
    stats = srv.stats()
    assert stats.requests_failed == 1 and stats.requests_done == 2


def test_cancelled_requests_leave_and_the_others_are_untouched():
    """A client that goes away: one request cancelled while queued (it never runs), one
    while active (evicted at the next tick, its range and slot reused by the queue); both
    end as VT_REQ_CANCELLED without a result, and the other requests keep their bits."""
    srv = vg.ClothServer(hbm_budget_bytes=1 << 30, max_cloths=2, substeps=3, iterations=4)
    plan = [(request(20, 0.5), 6), (request(24, 0.55), 9), (request(16, 0.6), 5), (request(18, 0.5), 4)]
    ids = []
    for spec, frames in plan:
        s = registered(spec)
        ids.append(srv.submit(s, frames))
        s.close()
    srv.tick()                 # two slots: requests 0 and 1 active, 2 and 3 queued
    srv.cancel(ids[2])         # queued: leaves at once
    assert srv.poll(ids[2])[0] == _abi.REQ_CANCELLED
    srv.tick()
    srv.cancel(ids[1])         # active: evicted by the next tick, request 3 takes its slot
    for _ in range(60):
        info = srv.tick()
        if info.active == 0 and info.queued == 0:
            break
    for k in (1, 2):
        assert srv.poll(ids[k])[0] == _abi.REQ_CANCELLED
        with pytest.raises(vg.VtError) as e:
            srv.result(ids[k])
        assert e.value.status == _abi.VT_ERR_STATE
        with pytest.raises(vg.VtError):
            srv.cancel(ids[k])  # already ended
    for k in (0, 3):
        spec, frames = plan[k]
        assert srv.poll(ids[k]) == (_abi.REQ_DONE, frames)
        assert np.array_equal(bits(srv.result(ids[k])), bits(alone(spec, frames)))
    stats = srv.stats()
    assert stats.requests_cancelled == 2 and stats.requests_done == 2 and stats.requests_failed == 0


def test_rejects_non_grid_and_oversize():
    srv = vg.ClothServer(hbm_budget_bytes=1 << 27, max_cloths=2)  # ~300k particles of arena
    s = vg.ClothSolver()
    verts, idx = W.grid_mesh(3, 0.06)
    s.add_cloth(verts, idx, np.eye(4), 0.03)
    with pytest.raises(vg.VtError) as e:
        srv.submit(s, 1)  # no grid constraint build: not a grid cloth
    assert e.value.status == _abi.VT_ERR_INVALID_ARGUMENT
    big = registered(request(700))  # 490k particles: more than a 128 MB arena holds
    with pytest.raises(vg.VtError) as e:
        srv.submit(big, 1)
    assert e.value.status == _abi.VT_ERR_CAPACITY


def test_admission_stops_on_a_budget_above_16_gb():
    """A 20 GiB budget with the particle cap off: 173 requests of 512 x 512 particles and
    a small one fill the arena (45.5 M particles; the arena's neighbour lists alone pass
    2^31 words, so the small request's list block starts beyond a 32-bit offset), the
    next request waits for memory, and the small request's result equals the same cloth
    alone."""
    budget = 20 << 30
    S, It = 2, 2
    srv = vg.ClothServer(hbm_budget_bytes=budget, max_cloths=256, max_active_particles=0, substeps=S,
                         iterations=It)
    per = 472  # device bytes per arena particle
    cap = (budget - 256 * 1860 - (1 << 20)) // per
    big = W.ClothSpec(512, 0.02, W.horizontal_cloth(512, 0.02, 0.8), [0, 511], request(16).colliders)
    n_big = cap // (512 * 512)
    assert n_big * 512 * 512 > (1 << 31) // 64, "the arena should pass the old 32-bit list offset"
    small = request(32, 0.45)
    ids = [submit_described(srv, big, 3) for _ in range(n_big)]
    rid_small = submit_described(srv, small, 3)
    rid_wait = submit_described(srv, big, 3)
    info = srv.tick()
    admitted = info.admitted
    for _ in range(3):  # uploads may spread admissions over ticks
        if srv.poll(rid_small)[0] == _abi.REQ_ACTIVE:
            break
        info = srv.tick()
        admitted += info.admitted
    assert srv.poll(rid_small)[0] in (_abi.REQ_ACTIVE, _abi.REQ_DONE)
    assert srv.poll(rid_wait)[0] == _abi.REQ_QUEUED, "the request beyond the budget should wait"
    assert admitted == n_big + 1
    assert srv.stats().bytes_in_use <= budget
    for _ in range(20):
        info = srv.tick()
        if srv.poll(rid_small)[0] == _abi.REQ_DONE and srv.poll(ids[-1])[0] == _abi.REQ_DONE:
            break
    assert srv.poll(rid_small) == (_abi.REQ_DONE, 3)
    assert np.array_equal(bits(srv.result(rid_small)), bits(alone(small, 3, S, It)))
    srv.close()
