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


# The numpy restatements of the workload generators live with the oracle
# (bench.py's CPU arm uses them too).
from pyoracle import GAMMA, lattice as lattice_np, mix64  # noqa: E402,F401


def header_functions(path=os.path.join(INCLUDE, "sphx.h")):
    """Names of the functions a C header declares (sphx_* identifiers
    followed by an opening parenthesis outside comments)."""
    import re
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    return sorted(set(re.findall(r"\b(sphx_[a-z0-9_]+)\s*\(", src)))
