"""GPU parity of the sm_103a step against the oracle and the golden fixtures.

Every call goes through the C-ABI (libsphx.so via ctypes).  The bar:
  * integer work (cells, hashes, accepted-neighbour multisets) bit-exact;
  * density, pressure, force and acceleration after one step within
    REL_TOL = 1e-5 of the reference's FP32 update(), metric rel_err (max over
    particles of |x - y| / max(|y|, rms|y|));
  * integration and wall reflection bit-exact given the step's own force
    and density.
"""
import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu

CONFIG_ARGS = np.array([0.125, 1000.0, 20.0, 1.0, 0.1, -9.8, 0.0], np.float32)


def bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def settings_from(sphx, args):
    return sphx.Settings(*[float(x) for x in args])


def scene(sphx, args, pos, vel=None, box=None, **opt):
    return sphx.Scene(settings_from(sphx, args), box if box is not None else sphx.reference_box(),
                      pos, vel, sphx.default_options(**opt))


def accel(force, rho, g):
    a = force / rho[:, None]
    a[:, 1] += g
    return a


def golden_by_id(g):
    n = len(g["ids"])
    out = {}
    for f in ("pos", "vel", "rho", "prs", "force", "hash"):
        a = np.zeros_like(g[f])
        a[g["ids"]] = g[f]
        out[f] = a
    return out


@pytest.mark.parametrize("name", ["step_block", "step_refscene", "step_origin"])
@pytest.mark.parametrize("use_graph", [0, 1])
def test_one_step_vs_reference_golden(sphx_lib, golden, name, use_graph):
    g = golden(name)
    ref = golden_by_id(g)
    with scene(sphx_lib, g["args"], g["pos_in"], g["vel_in"], use_graph=use_graph) as sc:
        sc.step(float(g["dt"]), 1)
        out = sc.read()
    assert rel_err(out["rho"], ref["rho"]) < REL_TOL
    assert rel_err(out["prs"], ref["prs"]) < REL_TOL
    assert rel_err(out["force"], ref["force"]) < REL_TOL
    gval = float(g["args"][5])
    assert rel_err(accel(out["force"], out["rho"], gval), accel(ref["force"], ref["rho"], gval)) < REL_TOL
    assert rel_err(out["pos"], ref["pos"]) < REL_TOL
    assert rel_err(out["vel"], ref["vel"]) < REL_TOL


@pytest.mark.parametrize("name", ["block", "refscene", "origin"])
def test_neighbor_multisets_bit_exact_vs_reference(sphx_lib, golden, name):
    g = golden("digest_" + name)
    args = CONFIG_ARGS.copy()
    args[4] = g["h"]
    with scene(sphx_lib, args, g["pos"]) as sc:
        cnt, dig = sc.neighbor_digest()
    assert np.array_equal(cnt, g["count"])
    assert np.array_equal(dig, g["digest"])


def test_cells_and_hashes_bit_exact(sphx_lib, port):
    rng = np.random.default_rng(5)
    pos = np.concatenate([rng.uniform(-3, 3, (5000, 3)),
                          rng.integers(-30, 30, (500, 3)) * 0.1,
                          rng.uniform(-0.15, 0.15, (500, 3))]).astype(np.float32)
    with scene(sphx_lib, CONFIG_ARGS, pos) as sc:
        cells, hsh = sc.cells()
    exp = np.array([port.cell(*p, np.float32(0.1)) for p in pos], np.int32)
    assert np.array_equal(cells, exp)
    exp_h = np.array([port.hash16(*c) for c in exp], np.uint16)
    assert np.array_equal(hsh, exp_h)


def integrate_np(pos, vel, force, rho, args, box, dt):
    """numpy float32 restatement of sph.cpp:133-176 (per-axis bounds)."""
    f32 = np.float32
    h, g = f32(args[4]), f32(args[5])
    dt = f32(dt)
    x, v = pos.astype(f32).copy(), vel.astype(f32).copy()
    a = force / rho[:, None]
    a[:, 0] = a[:, 0] + f32(0)
    a[:, 1] = a[:, 1] + g
    a[:, 2] = a[:, 2] + f32(0)
    v = v + a * dt
    x = x + v * dt
    ylo = f32(box.ymin) + h
    xlo, xhi = h + f32(box.xmin), f32(box.xmax) - h
    zlo, zhi = h + f32(box.zmin), f32(box.zmax) - h
    off, damp = f32(box.offset), f32(box.damping)
    m = x[:, 1] < ylo
    x[m, 1] = (-x[m, 1] + f32(2) * ylo) + off
    v[m, 1] = -v[m, 1] * damp
    if box.has_ceiling:  # the optional ceiling, after the floor
        yhi = f32(box.ymax) - h
        m = x[:, 1] > yhi
        x[m, 1] = (-x[m, 1] + f32(2) * yhi) - off
        v[m, 1] = -v[m, 1] * damp
    for ax, lo, hi in ((0, xlo, xhi), (2, zlo, zhi)):
        m = x[:, ax] < lo
        x[m, ax] = (-x[m, ax] + f32(2) * lo) + off
        v[m, ax] = -v[m, ax] * damp
        m = x[:, ax] > hi
        x[m, ax] = (-x[m, ax] + f32(2) * hi) - off
        v[m, ax] = -v[m, ax] * damp
    return x, v


def test_integration_and_walls_bit_exact(sphx_lib):
    pos, box = sphx_lib.dambreak(12, box_dims=(1.2, 1.0, 1.2))
    rng = np.random.default_rng(2)
    vel = rng.normal(0, 3.0, pos.shape).astype(np.float32)  # drives particles into walls
    with scene(sphx_lib, CONFIG_ARGS, pos, vel, box=box) as sc:
        sc.step(0.002, 1)
        out = sc.read()
    x, v = integrate_np(pos, vel, out["force"], out["rho"], CONFIG_ARGS, box, 0.002)
    assert np.array_equal(bits(out["pos"]), bits(x))
    assert np.array_equal(bits(out["vel"]), bits(v))
    assert (x[:, 0] > box.xmin).all()


def test_ceiling_bit_exact(sphx_lib, port):
    """The optional ceiling (not in the reference's box) reflects like the
    floor; integration stays bit-exact, and the step matches the oracle's
    with the same ceiling."""
    pos, box = sphx_lib.dambreak(12, box_dims=(1.2, 1.0, 1.2))
    pos[:, 1] += np.float32(0.3)            # the block's top near the ceiling
    box.ymax, box.has_ceiling = 1.0, 1
    vel = np.random.default_rng(7).normal(0, 3.0, pos.shape).astype(np.float32)
    vel[:, 1] = np.abs(vel[:, 1])           # upwards
    with scene(sphx_lib, CONFIG_ARGS, pos, vel, box=box) as sc:
        sc.step(0.002, 1)
        out = sc.read()
    x, v = integrate_np(pos, vel, out["force"], out["rho"], CONFIG_ARGS, box, 0.002)
    assert np.array_equal(bits(out["pos"]), bits(x))
    assert np.array_equal(bits(out["vel"]), bits(v))
    assert (out["pos"][:, 1] <= np.float32(0.9) + np.float32(1e-3)).all()
    assert (out["vel"][:, 1] < 0).sum() > 0  # some bounced
    r = port.step(pos, vel, CONFIG_ARGS, 0.002, box=box.as_array()).by_id()
    for f in ("rho", "prs", "force", "pos", "vel"):
        assert rel_err(out[f], getattr(r, f)) < REL_TOL, f


def test_transforms_match_reference(sphx_lib, golden):
    g = golden("step_block")
    with scene(sphx_lib, g["args"], g["pos_in"], g["vel_in"]) as sc:
        sc.step(float(g["dt"]), 1)
        tr = sc.transforms()
        out = sc.read()
    ids = g["ids"][:64]
    exp = g["transforms"]
    # scale(h/2) part is exact; translation equals the particle's position
    assert np.array_equal(tr[ids][:, :12], exp[:, :12])
    assert np.array_equal(tr[:, 15], np.ones(len(tr), np.float32))
    assert np.array_equal(tr[:, 12:15], out["pos"] + np.float32(0))
    assert rel_err(tr[ids][:, 12:15], exp[:, 12:15]) < REL_TOL


def test_config0_scene_vs_oracle(sphx_lib, port):
    pos, box = sphx_lib.dambreak(15, box_dims=(1.0, 1.0, 1.0))
    vel = np.random.default_rng(8).normal(0, 0.5, pos.shape).astype(np.float32)
    r = port.step(pos, vel, CONFIG_ARGS, 0.002, box=box.as_array()).by_id()
    with scene(sphx_lib, CONFIG_ARGS, pos, vel, box=box) as sc:
        sc.step(0.002, 1)
        out = sc.read()
        cnt, dig = sc.neighbor_digest()
    for f in ("rho", "prs", "force", "pos", "vel"):
        assert rel_err(out[f], getattr(r, f)) < REL_TOL, f
    c2, d2 = port.neighbor_digest(out["pos"], 0.1)
    assert np.array_equal(cnt, c2) and np.array_equal(dig, d2)


def test_against_fp64_oracle(sphx_lib, port):
    """Both FP32 implementations against the FP64 evaluation of the same sets."""
    pos, box = sphx_lib.dambreak(14, box_dims=(1.0, 1.0, 1.0), seed=3)
    vel = np.random.default_rng(1).normal(0, 0.5, pos.shape).astype(np.float32)
    rho64, prs64, f64 = port.fields_f64(pos, vel, CONFIG_ARGS)
    r = port.step(pos, vel, CONFIG_ARGS, 0.002, box=box.as_array()).by_id()
    with scene(sphx_lib, CONFIG_ARGS, pos, vel, box=box) as sc:
        sc.step(0.002, 1)
        out = sc.read()
    for name, gpu, ref, exact in (("rho", out["rho"], r.rho, rho64), ("prs", out["prs"], r.prs, prs64),
                                  ("force", out["force"], r.force, f64)):
        e_gpu, e_ref = rel_err(gpu, exact), rel_err(ref, exact)
        print("%s: gpu-vs-f64 %.2e  ref-vs-f64 %.2e" % (name, e_gpu, e_ref))
        assert e_gpu < REL_TOL and e_gpu <= max(2 * e_ref, 1e-6)


@pytest.mark.parametrize("R,slots", [(1, 256), (4, 256), (1, 1), (4, 1)])
def test_aliased_tiny_grid_is_exact(sphx_lib, port, R, slots):
    """A 5x5x5 cell grid far smaller than the scene: slots alias, results don't
    change.  Two of its five x columns are the grid's seam, whose particles
    walk alone; with a one-entry list they walk in the force pass too."""
    pos, box = sphx_lib.dambreak(16, box_dims=(2.0, 2.0, 2.0), seed=4)
    vel = np.random.default_rng(3).normal(0, 0.5, pos.shape).astype(np.float32)
    r = port.step(pos, vel, CONFIG_ARGS, 0.002, box=box.as_array()).by_id()
    with scene(sphx_lib, CONFIG_ARGS, pos, vel, box=box, grid_dims=(5, 5, 5),
               grid_origin=(-3, 0, 2), reorder_interval=R, neighbor_slots=slots) as sc:
        cnt, dig = sc.neighbor_digest()
        sc.step(0.002, 1)
        out = sc.read()
    c2, d2 = port.neighbor_digest(pos, 0.1)
    assert np.array_equal(cnt, c2) and np.array_equal(dig, d2)
    for f in ("rho", "prs", "force", "pos", "vel"):
        assert rel_err(out[f], getattr(r, f)) < REL_TOL, f


def test_aliased_tiny_grid_list_and_walk_agree(sphx_lib):
    """On the aliased grid the seam particles' force comes from their list or
    from the walk of the force pass's deferred particles: the same bits."""
    pos, box = sphx_lib.dambreak(16, box_dims=(2.0, 2.0, 2.0), seed=4)
    vel = np.random.default_rng(3).normal(0, 0.5, pos.shape).astype(np.float32)
    outs = []
    for slots in (1, 1024):
        with scene(sphx_lib, CONFIG_ARGS, pos, vel, box=box, grid_dims=(5, 5, 5),
                   grid_origin=(-3, 0, 2), neighbor_slots=slots) as sc:
            sc.step(0.002, 3)
            outs.append(sc.read())
    for f in ("rho", "prs", "force", "pos", "vel"):
        assert np.array_equal(outs[0][f], outs[1][f]), f


def test_dense_collision_region_digest(sphx_lib, port):
    """Random particles around the origin, where bucket collisions concentrate."""
    rng = np.random.default_rng(11)
    pos = rng.uniform(-1.2, 1.2, (30000, 3)).astype(np.float32)
    with scene(sphx_lib, CONFIG_ARGS, pos) as sc:
        cnt, dig = sc.neighbor_digest()
    c2, d2 = port.neighbor_digest(pos, 0.1)
    assert np.array_equal(cnt, c2) and np.array_equal(dig, d2)


@pytest.mark.parametrize("slots", [256, 1])
def test_collision_region_step_vs_oracle(sphx_lib, port, slots):
    """A step in the bucket-collision region around the origin.  Particles
    whose 27-cell neighbourhood has a collision take the per-particle walk
    with bucket weights, in the kernels that follow the density and force
    passes; with a one-entry list every particle walks in the force pass."""
    rng = np.random.default_rng(11)
    pos = rng.uniform(-1.2, 1.2, (30000, 3)).astype(np.float32)
    cells = np.trunc(pos / np.float32(0.1)).astype(np.int64)
    L = sphx_lib.lib()
    flagged = sum(1 for c in np.unique(cells, axis=0)
                  if L.sphx_collision_flags(int(c[0]), int(c[1]), int(c[2]), 0) & 1)
    assert flagged > 0  # the scene exercises the collision walk
    with scene(sphx_lib, CONFIG_ARGS, pos, neighbor_slots=slots) as sc:
        sc.step(0.002, 1)
        out = sc.read()
    r = port.step(pos, None, CONFIG_ARGS, 0.002).by_id()
    for f in ("rho", "prs", "force", "pos", "vel"):
        assert rel_err(out[f], getattr(r, f)) < REL_TOL, f


def test_exact_lattice_on_cell_faces_digest(sphx_lib, port):
    """An unjittered lattice at spacing h/2 around the origin puts particles
    on (or a rounding away from) cell faces, across the double-width cell 0
    and the bucket-collision region: accepted multisets bit-exact, through
    the direct-addressed walk of a reordering step."""
    k = np.arange(-15, 16, dtype=np.float32) * np.float32(0.05)
    g = np.stack(np.meshgrid(k, k + np.float32(0.8), k, indexing="ij"), -1).reshape(-1, 3)
    pos = np.ascontiguousarray(g, dtype=np.float32)
    with scene(sphx_lib, CONFIG_ARGS, pos) as sc:
        cnt, dig = sc.neighbor_digest()
    c2, d2 = port.neighbor_digest(pos, 0.1)
    assert np.array_equal(cnt, c2) and np.array_equal(dig, d2)
    assert cnt.max() > 0


@pytest.mark.parametrize("R", [1, 4, 16])
def test_multi_step_vs_oracle(sphx_lib, port, R):
    pos, box = sphx_lib.dambreak(12, box_dims=(1.0, 1.0, 1.0), seed=6)
    p0, v0, _, _ = port.run(pos, None, CONFIG_ARGS, 0.002, 5, box=box.as_array())
    with scene(sphx_lib, CONFIG_ARGS, pos, box=box, reorder_interval=R) as sc:
        sc.step(0.002, 5)
        out = sc.read()
    assert rel_err(out["pos"], p0) < REL_TOL
    assert rel_err(out["vel"], v0) < 1e-3  # 5 chained steps: rounding grows, stays small


def test_single_particle(sphx_lib, port):
    pos = np.array([[0.05, 0.5, -0.05]], np.float32)
    r = port.step(pos, None, CONFIG_ARGS, 0.002).by_id()
    with scene(sphx_lib, CONFIG_ARGS, pos) as sc:
        sc.step(0.002, 1)
        out = sc.read()
    assert np.array_equal(bits(out["rho"]), bits(r.rho))
    assert np.array_equal(bits(out["pos"]), bits(r.pos))
    assert np.array_equal(bits(out["vel"]), bits(r.vel))
