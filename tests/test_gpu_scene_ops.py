"""Scene initialisation on the device and runtime scene changes (the
reference GUI's RESET re-creates its system with new settings,
Tester.cpp:148-173)."""
import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu


def desc(sphx, n=(14, 9, 11), origin=(-0.45, 0.15, -0.4), seed=5):
    return sphx.LatticeDesc(n[0], n[1], n[2], (sphx.C.c_float * 3)(*origin), sphx.SPACING,
                            sphx.JITTER, seed)


def test_device_lattice_is_bit_identical_to_host(sphx_lib):
    sphx = sphx_lib
    d = desc(sphx)
    host = sphx.lattice(d.nx, d.ny, d.nz, tuple(d.origin), d.spacing, d.jitter, d.seed)
    s = sphx.config_settings()
    box = sphx.Box(-1, 1, 0, 2, -1, 1, 0.5, 0.0001, 0)
    with sphx.Scene.from_lattice(s, box, d) as sc:
        out = sc.read()
        assert np.array_equal(out["pos"], host) and not out["vel"].any()
        sc.step(sphx.DT, 5)
        dev = sc.read()
    with sphx.Scene(s, box, host) as sc:
        sc.step(sphx.DT, 5)
        ref = sc.read()
    for f in ("pos", "vel", "rho", "prs", "force"):
        assert np.array_equal(dev[f], ref[f]), f


def test_replace_scene_keeps_the_others(sphx_lib):
    sphx = sphx_lib
    scenes = sphx.batch_scenes(count=3, seed=21, nmin=500, nmax=4000)
    new_s = sphx.config_settings(35.0, 2.5)
    new_pos, new_box = sphx.dambreak(9, 7, 8, seed=77)
    with sphx.Scene.batch(scenes) as b:
        b.step(sphx.DT, 3)
        b.replace_scene(1, new_s, new_box, new_pos)
        b.step(sphx.DT, 4)
        got = [b.read_scene(k) for k in range(3)]
    for k in (0, 2):
        s, pos, box = scenes[k]
        with sphx.Scene(s, box, pos) as one:
            one.step(sphx.DT, 7)
            ref = one.read()
        for f in ("pos", "vel", "rho"):
            assert np.array_equal(got[k][f], ref[f]), (k, f)
    with sphx.Scene(new_s, new_box, new_pos) as one:
        one.step(sphx.DT, 4)
        ref = one.read()
    for f in ("pos", "vel", "rho"):
        assert np.array_equal(got[1][f], ref[f]), f


def test_replace_with_device_lattice(sphx_lib):
    sphx = sphx_lib
    scenes = sphx.batch_scenes(count=2, seed=4, nmin=500, nmax=3000)
    d = desc(sphx, n=(8, 8, 8), origin=(-0.3, 0.15, -0.3), seed=9)
    s = sphx.config_settings(15.0, 1.5)
    box = sphx.Box(-1, 1, 0, 2, -1, 1, 0.5, 0.0001, 0)
    with sphx.Scene.batch(scenes) as b:
        b.replace_scene(0, s, box, lattice=d)
        got = b.read_scene(0)
    host = sphx.lattice(8, 8, 8, (-0.3, 0.15, -0.3), sphx.SPACING, sphx.JITTER, 9)
    assert np.array_equal(got["pos"], host)


def test_settings_change_matches_fresh_scene(sphx_lib):
    sphx = sphx_lib
    pos, box = sphx.dambreak(12, box_dims=(1.2, 1.0, 1.2), seed=2)
    s0 = sphx.config_settings(20.0, 1.0)
    s1 = sphx.config_settings(32.0, 2.0)
    with sphx.Scene(s0, box, pos) as sc:
        sc.step(sphx.DT, 3)
        mid = sc.read()
        sc.set_settings(0, s1)
        sc.step(sphx.DT, 2)
        got = sc.read()
    with sphx.Scene(s1, box, mid["pos"], mid["vel"]) as fresh:
        fresh.step(sphx.DT, 2)
        ref = fresh.read()
    for f in ("pos", "vel", "rho", "prs", "force"):
        assert rel_err(got[f], ref[f]) < REL_TOL, f
