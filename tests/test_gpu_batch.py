"""Batched form: many independent scenes of uneven sizes and settings in one
handle, every launch covering all of them.  Each scene must come out exactly
as it does alone (same grid, same walk order, same kernels), and the batch
must agree with the oracle."""
import os

import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu

FIELDS = ("pos", "vel", "rho", "prs", "force")


def mixed_scenes(sphx):
    scenes = sphx.batch_scenes(count=9, seed=3, nmin=200, nmax=6000)
    # one scene around the origin (dense bucket collisions) and one in the reference box
    pos, box = sphx.dambreak(11, box_dims=(1.0, 1.0, 1.0), seed=9)
    pos = pos - np.float32([0.0, 0.0, 0.0])
    scenes.insert(3, (sphx.config_settings(30.0, 2.0), pos, box))
    ref = sphx.reference_settings()
    scenes.append((ref, sphx.reference_scene(7, ref.h), sphx.reference_box()))
    return scenes


def test_batch_equals_each_scene_alone(sphx_lib):
    sphx = sphx_lib
    scenes = mixed_scenes(sphx)
    with sphx.Scene.batch(scenes) as b:
        assert b.scene_count == len(scenes)
        b.step(sphx.DT, 4)
        got = [b.read_scene(k) for k in range(len(scenes))]
        allst = b.read()
    for k, (s, pos, box) in enumerate(scenes):
        with sphx.Scene(s, box, pos) as one:
            one.step(sphx.DT, 4)
            ref = one.read()
        for f in FIELDS:
            assert np.array_equal(got[k][f], ref[f]), (k, f)
    # the concatenated readout is the scenes in order
    first = 0
    for k in range(len(scenes)):
        n = len(scenes[k][1])
        assert np.array_equal(allst["pos"][first:first + n], got[k]["pos"])
        first += n


def test_batch_set_state_round_trip(sphx_lib):
    """sphx_set_state on a batch: the scenes' uploads share one staging area
    and are ordered on the device (each scene's copies wait for the previous
    scene's upload kernel, with no host wait between them).  The state read
    back is the state set, bit for bit; the last step's outputs are cleared;
    and a step from it agrees with the batch that reached that state by
    stepping."""
    sphx = sphx_lib
    scenes = mixed_scenes(sphx)
    with sphx.Scene.batch(scenes) as b:
        b.step(sphx.DT, 3)
        st = b.read()
        b.step(sphx.DT, 1)
        cont = b.read()
    with sphx.Scene.batch(scenes) as b2:
        b2.step(sphx.DT, 1)  # outputs of an unrelated step, to be cleared
        b2.set_state(st["pos"], st["vel"])
        back = b2.read()
        for f in ("pos", "vel"):
            assert np.array_equal(back[f].view(np.uint32), st[f].view(np.uint32)), f
        for f in ("rho", "prs", "force"):
            assert not back[f].any(), f
        b2.step(sphx.DT, 1)
        nxt = b2.read()
    # storage orders differ (cell order of different steps): equal up to the
    # order of particles with equal x in one cell
    for f in FIELDS:
        assert rel_err(nxt[f], cont[f]) < 1e-6, f


def test_batch_vs_oracle(sphx_lib, port):
    sphx = sphx_lib
    scenes = mixed_scenes(sphx)
    with sphx.Scene.batch(scenes) as b:
        cnt, dig = b.neighbor_digest()
        b.step(sphx.DT, 1)
        got = [b.read_scene(k) for k in range(len(scenes))]
    first = 0
    for k, (s, pos, box) in enumerate(scenes):
        n = len(pos)
        c2, d2 = port.neighbor_digest(pos, s.h)
        assert np.array_equal(cnt[first:first + n], c2) and np.array_equal(dig[first:first + n], d2)
        r = port.step(pos, None, sphx.args_array(s), sphx.DT, box=box.as_array()).by_id()
        for f in ("rho", "prs", "force", "pos", "vel"):
            assert rel_err(got[k][f], getattr(r, f)) < REL_TOL, (k, f)
        first += n


def test_512_scene_benchmark_mix_vs_oracle(sphx_lib, port):
    """The batched benchmark's own 512 scenes (7.7M particles, counts
    log-uniform in [1000, 65536], per-scene k and mu): one batched step,
    every scene's fields and neighbour multisets against the oracle's step
    of that scene alone."""
    sphx = sphx_lib
    scenes = sphx.batch_scenes(512, seed=0)
    with sphx.Scene.batch(scenes) as b:
        cnt, dig = b.neighbor_digest()
        b.step(sphx.DT, 1)
        got = b.read()
        ranges = [b.scene_range(k) for k in range(len(scenes))]
    worst = {f: 0.0 for f in ("rho", "prs", "force", "pos", "vel")}
    for k, (s, pos, box) in enumerate(scenes):
        first, n = ranges[k]
        assert n == len(pos)
        c2, d2 = port.neighbor_digest(pos, s.h)
        assert np.array_equal(cnt[first:first + n], c2) and np.array_equal(dig[first:first + n], d2), k
        r = port.step(pos, None, sphx.args_array(s), sphx.DT, box=box.as_array()).by_id()
        for f in worst:
            e = rel_err(got[f][first:first + n], getattr(r, f))
            worst[f] = max(worst[f], e)
            assert e < REL_TOL, (k, f, e)
    print("512 scenes, worst error per field:", {f: "%.1e" % e for f, e in worst.items()})


def test_tuning_variants_agree(sphx_lib):
    sphx = sphx_lib
    scenes = mixed_scenes(sphx)
    outs = []
    for d, f in ((128, 256), (256, 128), (128, 128)):
        with sphx.Scene.batch(scenes) as b:
            b.set_tuning(d, f, 1)
            b.step(sphx.DT, 3)
            outs.append(b.read())
    for o in outs[1:]:
        for f in FIELDS:
            assert np.array_equal(o[f], outs[0][f]), f  # block size does not change the result


def test_autotune_and_cache(sphx_lib, tmp_path):
    sphx = sphx_lib
    scenes = mixed_scenes(sphx)
    cache = str(tmp_path / "tune.txt")
    with sphx.Scene.batch(scenes) as b:
        before = b.read()
        t = b.autotune(sphx.DT, trial_steps=2, cache_path=cache)
        assert t.density_threads in (128, 256) and t.force_threads in (128, 256)
        assert t.reorder_interval in (1, 2, 4) and t.ms_per_step > 0
        after = b.read()  # state restored after the trials
        for f in ("pos", "vel"):
            assert np.array_equal(before[f], after[f])
    assert os.path.exists(cache)
    with sphx.Scene.batch(scenes) as b:
        t2 = b.autotune(sphx.DT, trial_steps=2, cache_path=cache)  # cache hit
        assert (t2.density_threads, t2.force_threads, t2.reorder_interval) == \
            (t.density_threads, t.force_threads, t.reorder_interval)
