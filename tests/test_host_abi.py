"""Host-side checks of the product library that need no GPU: the C-ABI loads
and exports every function include/sphx.h declares, and the host utilities
(settings constants, hash, cell, lattice, reference scene, bucket-collision
test) agree bit for bit with the oracle."""
import ctypes as C
import itertools

import numpy as np
import pytest

from _util import header_functions, lattice_np


def bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def test_every_declared_symbol_is_exported(sphx_lib):
    L = sphx_lib.lib()
    names = header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_create_without_gpu_fails_loudly(sphx_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    pos, box = sphx_lib.dambreak(4, box_dims=(1, 1, 1))
    with pytest.raises(sphx_lib.SphxError) as e:
        sphx_lib.Scene(sphx_lib.config_settings(), box, pos)
    assert e.value.code == -2


def test_derive_matches_oracle(sphx_lib, port, golden):
    g = golden("settings")
    for a, c in zip(g["args"], g["consts"]):
        d = sphx_lib.derive(sphx_lib.Settings(*[float(x) for x in a]))
        got = np.array([getattr(d, f) for f, _ in sphx_lib.Derived._fields_[:13]], np.float32)
        assert np.array_equal(bits(got), bits(c[:13]))
        assert np.array_equal(bits(np.array(d.sphere_scale, np.float32)), bits(c[13:]))


def test_hash_and_cell_match_golden(sphx_lib, golden):
    g = golden("hash_cell")
    got = np.array([sphx_lib.hash18(*c) for c in g["cells"]], np.uint32)
    assert np.array_equal(got, g["hashes"])
    cells = np.array([sphx_lib.cell(*p, g["h"]) for p in g["pos"]], np.int32)
    assert np.array_equal(cells, g["pos_cells"])


def test_lattice_matches_numpy_restatement(sphx_lib):
    for (nx, ny, nz), origin, seed in [((7, 5, 3), (-0.35, 0.15, -0.35), 0),
                                       ((16, 16, 16), (-7.85, 0.15, -3.85), 123456789)]:
        a = sphx_lib.lattice(nx, ny, nz, origin, 0.05, 0.0025, seed)
        b = lattice_np(nx, ny, nz, origin, 0.05, 0.0025, seed)
        assert np.array_equal(bits(a), bits(b))
        # index i + nx*(j + ny*k); jitter within +-5% of the spacing
        k, rem = np.divmod(np.arange(nx * ny * nz), nx * ny)
        j, i = np.divmod(rem, nx)
        base = np.asarray(origin, np.float64) + np.stack([i, j, k], 1) * 0.05
        dev = a - base
        assert np.abs(dev).max() <= 0.0025 + 1e-6 and dev.std() > 0.001


def test_oracle_workloads_match_product(sphx_lib):
    """The oracle side's dam-break blocks and settings (what the CPU arm of
    bench.py builds without the product library) are the product's, bit for
    bit: the headline block's corner, a batched-workload block, a served one."""
    import pyoracle
    for dims, seed in [((12, 12, 12), 0), ((9, 20, 6), 100003 * 0 + 17), ((31, 7, 13), 7919 + 3)]:
        a, box_a = sphx_lib.dambreak(*dims, seed=seed)
        b, box_b = pyoracle.dambreak(*dims, seed=seed)
        assert np.array_equal(bits(a), bits(b))
        assert np.array_equal(bits(box_a.as_array()), bits(box_b))
    for k, mu in [(20.0, 1.0), (13.25, 2.5)]:
        assert np.array_equal(sphx_lib.args_array(sphx_lib.config_settings(k, mu)),
                              pyoracle.config_args(k, mu))


def test_reference_scene_matches_oracle(sphx_lib, port):
    for w, h in [(8, 0.15), (15, 0.15), (5, 0.1)]:
        assert np.array_equal(bits(sphx_lib.reference_scene(w, h)), bits(port.reference_scene(w, h)))


def brute_flags(cx, cy, cz, face_mask):
    """Exact bucket-collision facts of the 27 cells around (cx, cy, cz)."""
    import sphx
    H = [sphx.hash18(cx + x, cy + y, cz + z) & 0xFFFF
         for x, y, z in itertools.product((-1, 0, 1), repeat=3)]
    dup = len(set(H)) < 27
    faces = []
    for f in range(6):
        axis, step = f // 2, (2 if f & 1 else -2)
        hit = False
        if (face_mask >> f) & 1:
            for a, b in itertools.product((-1, 0, 1), repeat=2):
                c = [cx, cy, cz]
                c[axis] += step
                c[(axis + 1) % 3] += a
                c[(axis + 2) % 3] += b
                hit |= (sphx.hash18(*c) & 0xFFFF) in H
        faces.append(hit)
    return dup, faces


def test_collision_flags_exact(sphx_lib):
    L = sphx_lib.lib()
    rng = np.random.default_rng(0)
    # bucket collisions cluster near the origin (small products keep high bits
    # clear): about 0.8% of cells within +-12 have a duplicate bucket
    near = np.array(list(itertools.product(range(-10, 11), repeat=3)))
    cells = np.concatenate([near, rng.integers(-300, 300, (2000, 3)),
                            rng.integers(-2 ** 20, 2 ** 20, (1000, 3))])
    ndup = nface = 0
    for c in cells:
        dup, faces = brute_flags(*c, 0x3F)
        fl = L.sphx_collision_flags(int(c[0]), int(c[1]), int(c[2]), 0x3F)
        assert bool(fl & 1) == dup
        for f in range(6):
            assert bool((fl >> (1 + f)) & 1) == faces[f], (c, f)
        ndup += dup
        nface += any(faces)
    assert ndup > 0 and nface > 0  # the sample exercises both cases
    # faces outside the mask are never reported
    for c in cells[:500]:
        assert L.sphx_collision_flags(int(c[0]), int(c[1]), int(c[2]), 0) & 0x7E == 0


def test_reference_presets(sphx_lib):
    s = sphx_lib.reference_settings()
    assert np.allclose(sphx_lib.args_array(s), [0.02, 1000, 1, 1.04, 0.15, -9.8, 0.2])
    b = sphx_lib.reference_box()
    assert (b.xmin, b.xmax, b.ymin, b.zmin, b.zmax, b.has_ceiling) == (-8, 8, 0, -8, 8, 0)
    assert np.float32(b.damping) == np.float32(0.5) and np.float32(b.offset) == np.float32(1e-4)
    o = sphx_lib.default_options()
    assert o.reorder_interval == 1 and o.max_cell_occupancy == 16384
    assert o.density_threads == 128 and o.force_threads == 128
    assert o.neighbor_slots == 256


def test_neighbor_slots_bound(sphx_lib):
    """A list longer than 1024 is refused before any device work."""
    opt = sphx_lib.default_options(neighbor_slots=1025)
    with pytest.raises(sphx_lib.SphxError) as e:
        sphx_lib.Scene(sphx_lib.reference_settings(), sphx_lib.reference_box(),
                       np.zeros((8, 3), np.float32), None, opt)
    assert e.value.code == -1 and "neighbor_slots" in str(e.value)
