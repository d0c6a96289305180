"""GPU: headless particle rendering (vt_solver_render / vt_batch_render) against the
oracle's restatement of the same sphere-impostor arithmetic, pixel for pixel."""
import numpy as np
import pytest

import oracle
import velvet_gb300 as vg
from velvet_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def simulated(spec, frames=3):
    s = vg.ClothSolver()
    W.build_plain(spec, s)
    for f in range(frames):
        s.update_colliders(spec.colliders(f))
        s.simulate(float(W.FRAME_DT), 5, 10, 1.0, 0.1, 0.06, spec.particle_diameter())
    s.sync()
    return s


@pytest.mark.parametrize("size", [(160, 120), (97, 61)])
def test_solver_render_matches_the_oracle(size):
    spec = W.ClothSpec(24, 0.02, W.horizontal_cloth(24, 0.02, 0.5), [0, 23], W.small().cloths[0].colliders)
    s = simulated(spec)
    rp = vg.render_params(size[0], size[1], eye=(0.4, 0.9, 0.9), target=(0, 0.4, 0),
                          particle_radius=spec.particle_diameter() / 2)
    got = s.render(rp)
    want = oracle.render(s.positions(), rp)
    assert np.array_equal(got, want), f"{(got != want).sum()} pixels differ"
    assert (got != rp.background).sum() > 100  # the cloth is in view


def test_batch_render_draws_every_cloth_and_occludes():
    specs = [W.ClothSpec(12, 0.02, W.horizontal_cloth(12, 0.02, h), [0, 11], W.small().cloths[0].colliders)
             for h in (0.45, 0.55)]
    solvers = [vg.ClothSolver() for _ in specs]
    b = vg.BatchSolver()
    for s, spec in zip(solvers, specs):
        W.build_plain(spec, s)
        b.add(s)
    b.simulate(float(W.FRAME_DT), 5, 10, 1.0, 0.1, 0.06)
    b.sync()
    rp = vg.render_params(128, 96, eye=(0.0, 1.2, 0.6), target=(0, 0.4, 0),
                          particle_radius=specs[0].particle_diameter() / 2)
    got = b.render(rp)
    pos = np.concatenate([b.positions(k) for k in range(len(specs))])
    assert np.array_equal(got, oracle.render(pos, rp))


def test_render_rejects_bad_parameters_and_unsimulated_solvers():
    spec = W.ClothSpec(8, 0.02, W.horizontal_cloth(8, 0.02, 0.5), [0, 7], W.small().cloths[0].colliders)
    s = vg.ClothSolver()
    W.build_plain(spec, s)
    rp = vg.render_params(32, 32, eye=(0, 1, 1), target=(0, 0.5, 0), particle_radius=0.01)
    with pytest.raises(vg.VtError):
        s.render(rp)  # nothing on the device yet
    s.simulate(float(W.FRAME_DT), 2, 2, 1.0, 0.1, 0.06, spec.particle_diameter())
    rp.particle_radius = 0.0
    with pytest.raises(vg.VtError):
        s.render(rp)
