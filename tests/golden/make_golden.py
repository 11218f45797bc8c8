"""Generates the golden fixtures in tests/golden/ from the reference's own CPU
code, compiled headless by oracle/build_oracle.py (oracle/_ref/libsphref.so).

Run where the reference checkout exists:  python tests/golden/make_golden.py
The fixtures pin the oracle restatement (and, through it, the GPU path) to
the reference without needing the reference at test time.

Contents (all little-endian numpy, .npz):
  hash_cell.npz   cell triples (incl. negatives and 32-bit overflow) -> the
                  reference getHash; positions (incl. negatives, exact
                  multiples of h, values near 0) -> getCell
  settings.npz    SPHSettings-derived constants for several constructor tuples
  step_*.npz      one updateParticlesCPU call: inputs and every output field
  digest_*.npz    accepted-neighbour fingerprints of the reference walk
  rollout.npz     10 chained reference steps on a small dam-break block
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import pyoracle  # noqa: E402
from _util import lattice_np  # noqa: E402

CONFIG_ARGS = np.array([0.125, 1000.0, 20.0, 1.0, 0.1, -9.8, 0.0], np.float32)
TESTER_ARGS = np.array([0.02, 1000.0, 1.0, 1.04, 0.15, -9.8, 0.2], np.float32)


def block(n, origin, seed):
    return lattice_np(n, n, n, origin, 0.05, 0.0025, seed)


def main():
    pyoracle.build()
    R = pyoracle.Ref()

    # hash / cell
    rng = np.random.default_rng(7)
    cells = np.concatenate([
        np.stack(np.meshgrid(np.arange(-6, 7), np.arange(-6, 7), np.arange(-6, 7), indexing="ij"), -1).reshape(-1, 3),
        rng.integers(-3000, 3000, (2000, 3)),
        rng.integers(-(2 ** 30), 2 ** 30, (500, 3)),
        np.array([[26, 27, 28], [-27, -26, -25], [2 ** 31 - 1, -(2 ** 31), 0]]),
    ]).astype(np.int32)
    hashes = np.array([R.get_hash(*c) for c in cells], np.uint32)
    h = np.float32(0.1)
    pos = np.concatenate([
        rng.uniform(-5, 5, (2000, 3)),
        (rng.integers(-50, 50, (300, 3)) * 0.1),
        rng.uniform(-0.2, 0.2, (300, 3)),
        np.array([[-0.1, 0.1, -0.0], [-1e-8, 1e-8, 0.09999999], [-0.19999999, 0.2, 0.3]]),
    ]).astype(np.float32)
    pcells = np.array([R.get_cell(*p, h) for p in pos], np.int32)
    np.savez_compressed(os.path.join(HERE, "hash_cell.npz"), cells=cells, hashes=hashes,
                        h=np.float32(h), pos=pos, pos_cells=pcells)

    # settings
    argsets = np.array([CONFIG_ARGS, TESTER_ARGS, [1.0, 998.0, 3.0, 0.5, 0.0457, -9.81, 0.0],
                        [0.3, 500.0, 40.0, 3.0, 0.25, -1.0, 0.1]], np.float32)
    consts = np.array([R.settings(a) for a in argsets], np.float32)
    np.savez_compressed(os.path.join(HERE, "settings.npz"), args=argsets, consts=consts)

    # one-step fixtures
    cases = {
        # config-0 style block (10^3) near the reference box corner, random velocities
        "step_block": (block(10, (-7.85, 0.15, -7.85), 11), 0.3, CONFIG_ARGS, 0.002),
        # the reference's own initParticles scene (width 8) with Tester settings, dt 0.003
        "step_refscene": (pyoracle.Port().reference_scene(8, 0.15), 0.0, TESTER_ARGS, 0.003),
        # a block straddling the origin (truncated cell 0 is two cells wide)
        "step_origin": (block(9, (-0.2, 0.15, -0.2), 12), 0.1, CONFIG_ARGS, 0.002),
    }
    for name, (p, vscale, args, dt) in cases.items():
        v = (np.random.default_rng(3).normal(0, 1, p.shape) * vscale).astype(np.float32)
        r = R.update_cpu(p, v, args, dt)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), pos_in=p, vel_in=v, args=args,
                            dt=np.float32(dt), ids=r.ids, pos=r.pos, vel=r.vel, rho=r.rho,
                            prs=r.prs, force=r.force, hash=r.hash, transforms=r.transforms[:64])
        cnt, dig = R.neighbor_digest(p, args[4])
        np.savez_compressed(os.path.join(HERE, "digest_" + name[5:] + ".npz"), pos=p,
                            h=np.float32(args[4]), count=cnt, digest=dig)

    # 10 chained reference steps, tracked by id
    p = block(8, (-7.85, 0.15, -7.85), 21)
    v = np.zeros_like(p)
    ids = np.arange(len(p), dtype=np.uint32)
    for _ in range(10):
        r = R.update_cpu(p, v, CONFIG_ARGS, 0.002)
        ids = ids[r.ids]
        p, v = r.pos, r.vel
    order = np.argsort(ids)
    np.savez_compressed(os.path.join(HERE, "rollout.npz"), pos_in=block(8, (-7.85, 0.15, -7.85), 21),
                        args=CONFIG_ARGS, dt=np.float32(0.002), steps=np.int32(10),
                        pos=p[order], vel=v[order])
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
