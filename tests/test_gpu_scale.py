"""Parity at the benchmark's own sizes: the 262,144-particle scene (64^3
block in an 8 x 4 x 4 m box), the 2,097,152-particle headline block (128^3,
16 x 8 x 8 m) and the 8,000,000-particle block (200^3, 25 x 12.5 x 12.5 m).
At each size one step's density, pressure, force, position and velocity are
compared with the oracle's step (the restatement of updateParticlesCPU,
src/sph.cpp:195-275) and the accepted-neighbour multisets with the oracle's
walk over the same positions.  Beside that, the size-independent checks:
results that must not change at all when only the storage order or the
reorder interval changes."""
import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu

CONFIG_ARGS = np.array([0.125, 1000.0, 20.0, 1.0, 0.1, -9.8, 0.0], np.float32)
FIELDS = ("pos", "vel", "rho", "prs", "force")


def settings(sphx):
    return sphx.Settings(*[float(x) for x in CONFIG_ARGS])


def test_262k_one_step_vs_oracle(sphx_lib, port):
    sphx = sphx_lib
    pos, box = sphx.dambreak(64, box_dims=(8.0, 4.0, 4.0))
    vel = np.random.default_rng(11).normal(0, 0.2, pos.shape).astype(np.float32)
    with sphx.Scene(settings(sphx), box, pos, vel) as sc:
        cnt, dig = sc.neighbor_digest()
        sc.step(0.002, 1)
        out = sc.read()
    c2, d2 = port.neighbor_digest(pos, 0.1)
    assert np.array_equal(cnt, c2) and np.array_equal(dig, d2)
    r = port.step(pos, vel, CONFIG_ARGS, 0.002, box=box.as_array()).by_id()
    for f in FIELDS:
        assert rel_err(out[f], getattr(r, f)) < REL_TOL, f


def one_step_vs_oracle(sphx, port, side, seed):
    """One step from the dam-break block with seeded random velocities (so
    that the viscosity term is exercised), every field against the oracle's
    step, plus the neighbour multisets of the initial positions."""
    pos, box = sphx.dambreak(side)
    vel = np.random.default_rng(seed).normal(0, 0.2, pos.shape).astype(np.float32)
    with sphx.Scene(settings(sphx), box, pos, vel) as sc:
        cnt, dig = sc.neighbor_digest()
        sc.step(0.002, 1)
        out = sc.read()
    c2, d2 = port.neighbor_digest(pos, 0.1)
    assert np.array_equal(cnt, c2) and np.array_equal(dig, d2)
    del c2, d2
    r = port.step(pos, vel, CONFIG_ARGS, 0.002, box=box.as_array()).by_id()
    errs = {f: rel_err(out[f], getattr(r, f)) for f in FIELDS}
    print("%d particles, one step against the oracle: %s"
          % (len(pos), {f: "%.1e" % e for f, e in errs.items()}))
    for f in FIELDS:
        assert errs[f] < REL_TOL, f
    # Both FP32 implementations against the FP64 evaluation of the same sums:
    # the GPU's error may not exceed twice the reference's own.
    rho64, prs64, f64 = port.fields_f64(pos, vel, CONFIG_ARGS)
    for name, gpu, ref, exact in (("rho", out["rho"], r.rho, rho64), ("prs", out["prs"], r.prs, prs64),
                                  ("force", out["force"], r.force, f64)):
        e_gpu, e_ref = rel_err(gpu, exact), rel_err(ref, exact)
        print("  %s: gpu-vs-f64 %.2e  ref-vs-f64 %.2e" % (name, e_gpu, e_ref))
        assert e_gpu <= max(2 * e_ref, 1e-6), name


def test_2m_one_step_fields_vs_oracle(sphx_lib, port):
    one_step_vs_oracle(sphx_lib, port, 128, 12)


def test_8m_one_step_fields_vs_oracle(sphx_lib, port):
    one_step_vs_oracle(sphx_lib, port, 200, 13)


def test_2m_neighbour_multisets_after_steps(sphx_lib, port):
    """After five steps of the headline scene, the GPU walk's accepted
    multisets equal the oracle's on the positions the GPU produced."""
    sphx = sphx_lib
    pos, box = sphx.dambreak(128)
    with sphx.Scene(settings(sphx), box, pos) as sc:
        sc.step(0.002, 5)
        p5 = sc.read()["pos"]
        cnt, dig = sc.neighbor_digest()
    c2, d2 = port.neighbor_digest(p5, 0.1)
    assert np.array_equal(cnt, c2) and np.array_equal(dig, d2)


def run_steps(sphx, pos, box, steps, **opt):
    with sphx.Scene(settings(sphx), box, pos, None, sphx.default_options(**opt)) as sc:
        sc.step(0.002, steps)
        return sc.read()


def distinct_x(pos):
    """The lattice puts four particles of a cell on one jittered column, and
    at float resolution some of them share x: the cell sort then orders
    them by storage index.  Raising each repeat to just above the value
    before it (in sorted order) makes every x distinct, so the sorted order
    is the same for every storage order."""
    pos = pos.copy()
    order = np.argsort(pos[:, 0], kind="stable")
    xs = pos[order, 0].tolist()
    f32 = np.float32
    for k in range(1, len(xs)):
        if xs[k] <= xs[k - 1]:
            xs[k] = float(np.nextafter(f32(xs[k - 1]), f32(np.inf)))
    pos[order, 0] = np.asarray(xs, np.float32)
    return pos


def compare(a, b, exact):
    for f in FIELDS:
        if exact:
            assert np.array_equal(a[f], b[f]), f
        else:
            assert rel_err(a[f], b[f]) < 1e-6, f


def test_2m_storage_order_invariance(sphx_lib):
    """Particles given in a shuffled order come out identical, by id: the
    cell sort's (x, index) order decides the walk, not the input order.
    Bit-identical after a step from distinct x; within 1e-6 after four steps,
    where equal x can reappear and be ordered by storage index."""
    sphx = sphx_lib
    pos, box = sphx.dambreak(128)
    pos = distinct_x(pos)
    perm = np.random.default_rng(3).permutation(len(pos))
    for steps, exact in ((1, True), (4, False)):
        a = run_steps(sphx, pos, box, steps)
        b = run_steps(sphx, pos[perm], box, steps)
        compare({f: a[f][perm] for f in FIELDS}, b, exact)


def test_2m_reorder_interval_invariance(sphx_lib):
    """Reordering the particle data every step or every 16 steps walks the
    same sorted order (directly or through the permutation): bit-identical
    over the first two steps from distinct x, within 1e-6 after six."""
    sphx = sphx_lib
    pos, box = sphx.dambreak(128)
    pos = distinct_x(pos)
    for steps, exact in ((2, True), (6, False)):
        a = run_steps(sphx, pos, box, steps, reorder_interval=1)
        b = run_steps(sphx, pos, box, steps, reorder_interval=16)
        compare(a, b, exact)


def test_8m_steps(sphx_lib):
    """The 8,000,000-particle block (200^3, 25 x 12.5 x 12.5 m) steps without
    error; its density field is that of the lattice (every particle has
    neighbours, none is empty)."""
    sphx = sphx_lib
    pos, box = sphx.dambreak(200)
    assert len(pos) == 8_000_000
    out = run_steps(sphx, pos, box, 2)
    assert np.isfinite(out["pos"]).all() and np.isfinite(out["force"]).all()
    self_density = sphx.derive(settings(sphx)).self_dens
    assert (out["rho"] > self_density).mean() > 0.999
