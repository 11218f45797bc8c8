"""Neighbour lists between the two walk kernels.  The density pass records
up to `neighbor_slots` accepted neighbours per particle; the force pass sums
over that list, or walks again (warp-cooperatively) for a particle with more.
Both routes visit the same neighbours in the same order through the same pair
arithmetic, so the step must be bit-identical whatever the list length, in
clumped fluid (most particles past any short list) and in the 2-neighbour
regime alike."""
import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu

CONFIG_ARGS = np.array([0.125, 1000.0, 20.0, 1.0, 0.1, -9.8, 0.0], np.float32)
FIELDS = ("pos", "vel", "rho", "prs", "force")


def clumped(seed=0):
    rng = np.random.default_rng(seed)
    core = rng.uniform(0.21, 0.33, (2500, 3))     # ~2 cells wide: hundreds of neighbours
    shell = rng.uniform(0.05, 0.6, (1500, 3))
    return np.concatenate([core, shell]).astype(np.float32)


def run(sphx, pos, slots, steps, reorder=1):
    s = sphx.Settings(*[float(x) for x in CONFIG_ARGS])
    opt = sphx.default_options(neighbor_slots=slots, reorder_interval=reorder)
    with sphx.Scene(s, sphx.reference_box(), pos, None, opt) as sc:
        sc.step(0.002, steps)
        return sc.read()


@pytest.mark.parametrize("reorder", [1, 3])
def test_list_length_does_not_change_results(sphx_lib, reorder):
    pos = clumped()
    outs = {k: run(sphx_lib, pos, k, 4, reorder) for k in (1, 16, 64, 1024)}
    for k in (1, 16, 1024):
        for f in FIELDS:
            assert np.array_equal(outs[k][f], outs[64][f]), (k, f)


def test_walking_force_matches_oracle(sphx_lib, port):
    """Every particle walks in the force pass (a one-entry list).  In a clump
    with hundreds of neighbours the pressure terms nearly cancel, so the
    force is judged as in the FP64 parity test: against the FP64 evaluation
    of the same neighbour sets, no worse than the reference's FP32 sum."""
    pos = clumped(seed=2)
    vel = np.random.default_rng(5).normal(0, 0.05, pos.shape).astype(np.float32)
    s = sphx_lib.Settings(*[float(x) for x in CONFIG_ARGS])
    opt = sphx_lib.default_options(neighbor_slots=1)
    with sphx_lib.Scene(s, sphx_lib.reference_box(), pos, vel, opt) as sc:
        sc.step(0.002, 1)
        out = sc.read()
    r = port.step(pos, vel, CONFIG_ARGS, 0.002).by_id()
    for f in ("rho", "prs"):
        assert rel_err(out[f], getattr(r, f)) < REL_TOL, f
    rho64, prs64, f64 = port.fields_f64(pos, vel, CONFIG_ARGS)
    e_gpu, e_ref = rel_err(out["force"], f64), rel_err(r.force, f64)
    print("force: gpu-vs-f64 %.2e  ref-vs-f64 %.2e  gpu-vs-ref %.2e"
          % (e_gpu, e_ref, rel_err(out["force"], r.force)))
    assert e_gpu < REL_TOL and e_gpu <= max(2 * e_ref, 1e-6)


def test_walk_stats_agree_with_digest(sphx_lib):
    """sphx_walk_stats counts what the walk does: its accepted visits are the
    digest's counts, every accepted pair was an r^2 test, and a uniform
    lattice spends a bounded number of tests per accepted pair."""
    pos, box = sphx_lib.dambreak(24, box_dims=(2.0, 2.0, 2.0), seed=5)
    s = sphx_lib.Settings(*[float(x) for x in CONFIG_ARGS])
    with sphx_lib.Scene(s, box, pos) as sc:
        tests, acc = sc.walk_stats()
        cnt, _ = sc.neighbor_digest()
    assert acc == int(cnt.sum())
    assert acc <= tests <= 8 * acc
