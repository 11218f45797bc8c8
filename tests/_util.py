"""Shared test helpers: paths, the parity metric and a numpy restatement of
the dam-break lattice generator (used to cross-check the product's)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "sph-fluid-simulator_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
INCLUDE = os.path.join(ROOT, "include")

for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)

# Parity tolerance for FP32 fields against the reference's FP32 update():
# max over particles of |x - y| / max(|y|, rms(|y|)), vectors compared by
# Euclidean norm.  The RMS floor keeps near-zero values (pressure near rest
# density, balanced forces) from turning rounding noise into huge ratios.
REL_TOL = 1e-5


def rel_err(x, y):
    x = np.asarray(x, np.float64).reshape(len(x), -1)
    y = np.asarray(y, np.float64).reshape(len(y), -1)
    d = np.linalg.norm(x - y, axis=1)
    ny = np.linalg.norm(y, axis=1)
    floor = np.sqrt(np.mean(ny ** 2))
    if floor == 0.0:
        return float(d.max())
    return float((d / np.maximum(ny, floor)).max())


GAMMA = np.uint64(0x9E3779B97F4A7C15)


def mix64(z):
    z = np.asarray(z, np.uint64)
    with np.errstate(over="ignore"):
        z = z + GAMMA
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def lattice_np(nx, ny, nz, origin, spacing, jitter, seed):
    """numpy restatement of sphx_lattice (float32 arithmetic, same order)."""
    n = nx * ny * nz
    idx = np.arange(n, dtype=np.uint64)
    k, rem = np.divmod(np.arange(n), nx * ny)
    j, i = np.divmod(rem, nx)
    ijk = [i, j, k]
    out = np.zeros((n, 3), np.float32)
    for a in range(3):
        with np.errstate(over="ignore"):
            ctr = np.uint64(seed) + (np.uint64(3) * idx + np.uint64(a)) * GAMMA
        r = mix64(ctr)
        u = (r >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)
        jit = (u * np.float32(2.0) - np.float32(1.0)) * np.float32(jitter)
        base = np.float32(origin[a]) + ijk[a].astype(np.float32) * np.float32(spacing)
        out[:, a] = base + jit
    return out


def header_functions(path=os.path.join(INCLUDE, "sphx.h")):
    """Names of the functions a C header declares (sphx_* identifiers
    followed by an opening parenthesis outside comments)."""
    import re
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    return sorted(set(re.findall(r"\b(sphx_[a-z0-9_]+)\s*\(", src)))
