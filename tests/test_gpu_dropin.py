"""sphx_update_particles — the reference's updateParticlesGPU contract over
60-byte Particle records (src/kernels/sphGPU.h:8-11) — against the oracle."""
import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu


def expected_hash(port, pos, h):
    return np.array([port.hash16(*port.cell(*p, np.float32(h))) for p in pos], np.uint16)


def test_one_call_matches_reference_step(sphx_lib, port):
    sphx = sphx_lib
    s = sphx.reference_settings()
    pos = sphx.reference_scene(10, s.h)
    vel = np.random.default_rng(0).normal(0, 0.2, pos.shape).astype(np.float32)
    rec = sphx.particles_from(pos, vel)
    acc_marker = np.random.default_rng(1).normal(0, 1, pos.shape).astype(np.float32)
    rec["acceleration"] = acc_marker
    tr = np.zeros((len(pos), 16), np.float32)
    sphx.update_particles(rec, s, 0.003, transforms=tr)
    r = port.step(pos, vel, sphx.args_array(s), 0.003).by_id()
    assert rel_err(rec["density"], r.rho) < REL_TOL
    assert rel_err(rec["pressure"], r.prs) < REL_TOL
    assert rel_err(rec["force"], r.force) < REL_TOL
    assert rel_err(rec["position"], r.pos) < REL_TOL
    assert rel_err(rec["velocity"], r.vel) < REL_TOL
    assert np.array_equal(rec["hash"], r.hash)  # hash of the pre-step cell, as the reference stores
    assert np.array_equal(rec["acceleration"], acc_marker)  # never written
    assert np.array_equal(tr[:, 12:15], rec["position"] + np.float32(0))
    assert np.all(tr[:, [0, 5, 10]] == np.float32(s.h / 2)) and np.all(tr[:, 15] == 1)
    sphx.release_update_particles()


def test_repeated_calls_follow_the_reference_rollout(sphx_lib, port):
    sphx = sphx_lib
    s = sphx.reference_settings()
    pos = sphx.reference_scene(8, s.h)
    rec = sphx.particles_from(pos)
    for _ in range(5):
        sphx.update_particles(rec, s, 0.003)
    p5, v5, _, _ = port.run(pos, None, sphx.args_array(s), 0.003, 5)
    assert rel_err(rec["position"], p5) < REL_TOL
    assert rel_err(rec["velocity"], v5) < 1e-3
    # a different particle count re-creates the cached state
    pos2 = sphx.reference_scene(6, s.h)
    rec2 = sphx.particles_from(pos2)
    sphx.update_particles(rec2, s, 0.003)
    r = port.step(pos2, None, sphx.args_array(s), 0.003).by_id()
    assert rel_err(rec2["density"], r.rho) < REL_TOL
    sphx.release_update_particles()
