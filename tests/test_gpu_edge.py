"""Edge cases of the GPU step: clumped cells (the reference's own physics
clumps at these parameters), error status raised by the kernels and
recovered from, invalid inputs, and 100-step rollout statistics."""
import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu

CONFIG_ARGS = np.array([0.125, 1000.0, 20.0, 1.0, 0.1, -9.8, 0.0], np.float32)


def scene(sphx, pos, vel=None, box=None, **opt):
    return sphx.Scene(sphx.Settings(*[float(x) for x in CONFIG_ARGS]),
                      box if box is not None else sphx.reference_box(), pos, vel,
                      sphx.default_options(**opt))


def clump(n_core=3000, n_shell=600, seed=0):
    rng = np.random.default_rng(seed)
    core = rng.uniform(0.205, 0.295, (n_core, 3))          # one cell: (2, 2, 2)
    shell = rng.uniform(0.05, 0.45, (n_shell, 3))
    return np.concatenate([core, shell]).astype(np.float32)


def test_large_cells_exact(sphx_lib, port):
    pos = clump()
    vel = np.random.default_rng(1).normal(0, 0.1, pos.shape).astype(np.float32)
    with scene(sphx_lib, pos, vel) as sc:
        cnt, dig = sc.neighbor_digest()
        sc.step(0.002, 1)
        out = sc.read()
    c2, d2 = port.neighbor_digest(pos, 0.1)
    assert cnt.max() > 3000
    assert np.array_equal(cnt, c2) and np.array_equal(dig, d2)
    r = port.step(pos, vel, CONFIG_ARGS, 0.002).by_id()
    for f in ("rho", "prs", "force"):
        assert rel_err(out[f], getattr(r, f)) < REL_TOL, f


def test_large_cells_deterministic(sphx_lib):
    pos = clump(seed=3)
    outs = []
    for _ in range(2):
        with scene(sphx_lib, pos) as sc:
            sc.step(0.002, 3)
            outs.append(sc.read())
    for f in ("pos", "vel", "rho"):
        assert np.array_equal(outs[0][f], outs[1][f])


def test_clumped_scene_batch_equals_alone(sphx_lib, port):
    """A clumped scene (a cell of 1,500 particles: large-cell sort, no lists,
    every particle walked again by the force pass) comes out bit-identical
    alone and beside another scene in a batch, and a step of it agrees with
    the oracle."""
    sphx = sphx_lib
    s = sphx.Settings(*[float(x) for x in CONFIG_ARGS])
    pos = clump(n_core=1500, n_shell=400, seed=5)
    vel = np.random.default_rng(6).normal(0, 0.1, pos.shape).astype(np.float32)
    box = sphx.reference_box()
    other, obox = sphx.dambreak(9, box_dims=(1.0, 1.0, 1.0), seed=2)
    with sphx.Scene(s, box, pos, vel) as one:
        one.step(0.002, 2)
        alone = one.read()
    with sphx.Scene.batch([(s, other, obox), (s, pos, box, vel)]) as b:
        b.step(0.002, 2)
        mixed = b.read_scene(1)
    for f in ("pos", "vel", "rho", "prs", "force"):
        assert np.array_equal(alone[f], mixed[f]), f
    with sphx.Scene(s, box, pos, vel) as one:
        one.step(0.002, 1)
        out = one.read()
    r = port.step(pos, vel, CONFIG_ARGS, 0.002).by_id()
    for f in ("rho", "prs", "force", "pos", "vel"):
        assert rel_err(out[f], getattr(r, f)) < REL_TOL, f


def test_cell_overflow_raises_then_recovers(sphx_lib):
    sphx = sphx_lib
    pos = clump(n_core=500, n_shell=0)
    with scene(sphx, pos, max_cell_occupancy=100) as sc:
        sc.step(0.002, 1)
        with pytest.raises(sphx.SphxError) as e:
            sc.synchronize()
        assert e.value.code == -5
        with pytest.raises(sphx.SphxError) as e:
            sc.step(0.002, 1)
        assert e.value.code == -6  # error state until the state is replaced
        spread = sphx.dambreak(8, box_dims=(1, 1, 1))[0]
        spread = np.concatenate([spread, spread[: len(pos) - len(spread)] + 0.001]) \
            if len(spread) < len(pos) else spread[: len(pos)]
        sc.set_state(spread)
        sc.step(0.002, 1)
        sc.synchronize()


def test_domain_error_midrun(sphx_lib):
    sphx = sphx_lib
    pos, box = sphx.dambreak(6, box_dims=(1, 1, 1))
    vel = np.zeros_like(pos)
    vel[5] = [3e38, 0, 0]  # overflows to inf after one integration
    with scene(sphx, pos, vel, box=box) as sc:
        sc.step(0.002, 3)
        with pytest.raises(sphx.SphxError) as e:
            sc.synchronize()
        assert e.value.code == -4
        sc.set_state(pos)
        sc.step(0.002, 2)
        sc.synchronize()


def test_set_state_keeps_storage_order_and_results(sphx_lib, port):
    """sphx_set_state writes the caller's (id-ordered) state into the rows the
    particles already occupy, so the step after it starts from the last
    step's cell order.  Its result equals a fresh scene's from the same state
    and the oracle's step, within the one-step tolerance (particles of one cell
    with equal x are ordered by storage position, so the last bits may move)."""
    sphx = sphx_lib
    pos, box = sphx.dambreak(14, box_dims=(1.0, 1.0, 1.0), seed=8)
    with scene(sphx, pos, box=box) as sc:
        sc.step(0.002, 6)
        st = sc.read()
        sc.set_state(st["pos"], st["vel"])
        back = sc.read()
        assert np.array_equal(back["pos"], st["pos"]) and np.array_equal(back["vel"], st["vel"])
        sc.step(0.002, 1)
        a = sc.read()
    with scene(sphx, st["pos"], st["vel"], box=box) as fresh:
        fresh.step(0.002, 1)
        b = fresh.read()
    r = port.step(st["pos"], st["vel"], CONFIG_ARGS, 0.002, box=box.as_array()).by_id()
    for f in ("pos", "vel", "rho", "prs", "force"):
        assert rel_err(a[f], b[f]) < 1e-6, f
        assert rel_err(a[f], getattr(r, f)) < REL_TOL, f


def test_invalid_inputs(sphx_lib):
    sphx = sphx_lib
    pos = np.zeros((4, 3), np.float32)
    pos[2, 1] = np.nan
    with pytest.raises(sphx.SphxError) as e:
        scene(sphx, pos)
    assert e.value.code == -4
    with pytest.raises(sphx.SphxError) as e:
        scene(sphx, np.zeros((0, 3), np.float32))
    assert e.value.code == -1
    bad = sphx.Settings(0.125, 1000, 20, 1, 0.0, -9.8, 0)
    with pytest.raises(sphx.SphxError):
        sphx.Scene(bad, sphx.reference_box(), np.ones((3, 3), np.float32))


def stats(pos, vel, rho, m=0.125):
    return {"mean_rho": float(np.mean(rho, dtype=np.float64)),
            "ke": float(0.5 * m * np.sum(vel.astype(np.float64) ** 2)),
            "com": pos.astype(np.float64).mean(axis=0)}


def test_rollout_100_steps_statistics(sphx_lib, port):
    """Trajectories are chaotic; the aggregates must stay close."""
    sphx = sphx_lib
    pos, box = sphx.dambreak(15, box_dims=(1.0, 1.0, 1.0))
    p_ref, v_ref, rho_ref, _ = port.run(pos, None, CONFIG_ARGS, 0.002, 100, box=box.as_array())
    with scene(sphx, pos, box=box) as sc:
        sc.step(0.002, 100)
        out = sc.read()
    a, b = stats(out["pos"], out["vel"], out["rho"]), stats(p_ref, v_ref, rho_ref)
    e_rho = abs(a["mean_rho"] - b["mean_rho"]) / b["mean_rho"]
    e_ke = abs(a["ke"] - b["ke"]) / b["ke"]
    e_com = float(np.linalg.norm(a["com"] - b["com"]))
    print("100-step drift: mean density %.2e, kinetic energy %.2e, centre of mass %.2e m"
          % (e_rho, e_ke, e_com))
    assert e_rho < 5e-3 and e_ke < 5e-2 and e_com < 5e-3


def test_set_state_rejects_out_of_domain(sphx_lib):
    """State replacement is validated on the device: the first bad row is
    named, stepping is refused until a valid state replaces it."""
    sphx = sphx_lib
    pos, box = sphx.dambreak(6, box_dims=(1, 1, 1))
    with scene(sphx, pos, box=box) as sc:
        sc.step(0.002, 1)
        bad = pos.copy()
        bad[17, 2] = np.inf
        bad[40, 0] = np.nan
        with pytest.raises(sphx.SphxError) as e:
            sc.set_state(bad)
        assert e.value.code == -4 and "position 17" in str(e.value)
        with pytest.raises(sphx.SphxError) as e:
            sc.step(0.002, 1)
        assert e.value.code == -6
        far = pos.copy()
        far[3, 1] = 0.1 * 2.0 ** 31  # cell quotient past 2^30
        with pytest.raises(sphx.SphxError) as e:
            sc.set_state(far)
        assert e.value.code == -4 and "position 3" in str(e.value)
        sc.set_state(pos)
        sc.step(0.002, 2)
        sc.synchronize()
