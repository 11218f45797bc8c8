"""ctypes bindings for the oracle libraries (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline /
reference arm import this module, as the checker; the product never does.

* :class:`Port` wraps ``oracle/_build/liboracle.so`` — the project's CPU
  restatement of the reference hot path (oracle/sph_oracle.cpp).
* :class:`Ref` wraps ``oracle/_ref/libsphref.so`` — the reference's own CPU
  code compiled headless (oracle/ref_harness.cpp); present only where the
  reference checkout was available to build it.

Positions / velocities are float32 arrays of shape (n, 3).  ``args`` is the
reference's SPHSettings constructor tuple (mass, restDensity, gasConst,
viscosity, h, g, tension) — SPHSystem.h:15-17.  ``box`` is None (the
reference's hard-coded box, sph.cpp:139-140) or a 9-float array
(xmin, xmax, ymin, ymax, zmin, zmax, damping, offset, has_ceiling).
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libsphref.so")

_f = np.ctypeslib.ndpointer(np.float32, flags="C")
_d = np.ctypeslib.ndpointer(np.float64, flags="C")
_u32 = np.ctypeslib.ndpointer(np.uint32, flags="C")
_u16 = np.ctypeslib.ndpointer(np.uint16, flags="C")
_u64 = np.ctypeslib.ndpointer(np.uint64, flags="C")
_vp = C.c_void_p

REFERENCE_BOX = None


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_vp)


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


class StepResult:
    """Post-step arrays in the implementation's output order; ``ids[k]`` is
    the input index of output row k."""

    def __init__(self, n):
        self.ids = np.zeros(n, np.uint32)
        self.pos = np.zeros((n, 3), np.float32)
        self.vel = np.zeros((n, 3), np.float32)
        self.rho = np.zeros(n, np.float32)
        self.prs = np.zeros(n, np.float32)
        self.force = np.zeros((n, 3), np.float32)
        self.hash = np.zeros(n, np.uint16)
        self.transforms = np.zeros((n, 16), np.float32)

    def by_id(self):
        """Returns a copy with rows reordered so that row i is input particle i."""
        n = len(self.ids)
        out = StepResult(n)
        for name in ("pos", "vel", "rho", "prs", "force", "hash", "transforms"):
            getattr(out, name)[self.ids] = getattr(self, name)
        out.ids[:] = np.arange(n, dtype=np.uint32)
        return out


class _Lib:
    prefix = ""

    def __init__(self, path):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        p = self.prefix
        L = self.lib
        getattr(L, p + "sizeof_particle").restype = C.c_int
        getattr(L, p + "settings").argtypes = [_f, _f]
        getattr(L, p + "neighbor_digest").argtypes = [C.c_size_t, _f, C.c_float, _u32, _u64]

    def settings(self, args):
        out = np.zeros(29, np.float32)
        getattr(self.lib, self.prefix + "settings")(_f32(args), out)
        return out

    def neighbor_digest(self, pos, h):
        pos = _f32(pos, (-1, 3))
        n = len(pos)
        cnt = np.zeros(n, np.uint32)
        dig = np.zeros(n, np.uint64)
        getattr(self.lib, self.prefix + "neighbor_digest")(n, pos, C.c_float(h), cnt, dig)
        return cnt, dig


class Ref(_Lib):
    """The reference's own CPU code (compiled headless)."""

    prefix = "ref_"

    def __init__(self, path=REF_PATH):
        super().__init__(path)
        L = self.lib
        L.ref_get_hash.restype = C.c_uint32
        L.ref_get_hash.argtypes = [C.c_int, C.c_int, C.c_int]
        L.ref_get_cell.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, _vp]
        L.ref_update_cpu.restype = C.c_int
        L.ref_update_cpu.argtypes = [C.c_size_t, _f, _vp, _f, C.c_float] + [_vp] * 8

    def get_hash(self, x, y, z):
        return self.lib.ref_get_hash(int(x), int(y), int(z))

    def get_cell(self, x, y, z, h):
        out = np.zeros(3, np.int32)
        self.lib.ref_get_cell(x, y, z, h, out.ctypes.data_as(_vp))
        return out

    def update_cpu(self, pos, vel, args, dt):
        pos = _f32(pos, (-1, 3))
        n = len(pos)
        vel = None if vel is None else _f32(vel, (n, 3))
        r = StepResult(n)
        rc = self.lib.ref_update_cpu(n, pos, _ptr(vel), _f32(args), C.c_float(dt),
                                     _ptr(r.ids), _ptr(r.pos), _ptr(r.vel), _ptr(r.rho),
                                     _ptr(r.prs), _ptr(r.force), _ptr(r.hash),
                                     _ptr(r.transforms))
        if rc != 0:
            raise RuntimeError("reference update failed: %d" % rc)
        return r


class Port(_Lib):
    """The project's CPU restatement of the reference hot path."""

    prefix = "orc_"

    def __init__(self, path=PORT_PATH):
        super().__init__(path)
        L = self.lib
        L.orc_hw_threads.restype = C.c_int
        for fn in ("orc_hash18", "orc_hash16"):
            getattr(L, fn).restype = C.c_uint32
            getattr(L, fn).argtypes = [C.c_int, C.c_int, C.c_int]
        L.orc_cell.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, _vp]
        L.orc_reference_scene.argtypes = [C.c_size_t, C.c_float, _f]
        L.orc_step.restype = C.c_int
        L.orc_step.argtypes = ([C.c_size_t, _f, _vp, _f, _vp, C.c_float, C.c_int, C.c_int]
                               + [_vp] * 8)
        L.orc_run.restype = C.c_int
        L.orc_run.argtypes = ([C.c_size_t, _f, _vp, _f, _vp, C.c_float, C.c_int, C.c_int]
                              + [_vp] * 4)
        L.orc_fields_f64.restype = C.c_int
        L.orc_fields_f64.argtypes = [C.c_size_t, _f, _vp, _f, _d, _d, _d]

    def hw_threads(self):
        return self.lib.orc_hw_threads()

    def hash18(self, x, y, z):
        return self.lib.orc_hash18(int(x), int(y), int(z))

    def hash16(self, x, y, z):
        return self.lib.orc_hash16(int(x), int(y), int(z))

    def cell(self, x, y, z, h):
        out = np.zeros(3, np.int32)
        self.lib.orc_cell(x, y, z, h, out.ctypes.data_as(_vp))
        return out

    def reference_scene(self, width, h):
        out = np.zeros((width ** 3, 3), np.float32)
        self.lib.orc_reference_scene(width, C.c_float(h), out)
        return out

    def step(self, pos, vel, args, dt, box=REFERENCE_BOX, threads=0, stable=False):
        pos = _f32(pos, (-1, 3))
        n = len(pos)
        vel = None if vel is None else _f32(vel, (n, 3))
        bx = None if box is None else _f32(box)
        r = StepResult(n)
        rc = self.lib.orc_step(n, pos, _ptr(vel), _f32(args), _ptr(bx), C.c_float(dt),
                               int(threads), int(bool(stable)), _ptr(r.ids), _ptr(r.pos),
                               _ptr(r.vel), _ptr(r.rho), _ptr(r.prs), _ptr(r.force),
                               _ptr(r.hash), _ptr(r.transforms))
        if rc != 0:
            raise RuntimeError("oracle step failed: %d" % rc)
        return r

    def run(self, pos, vel, args, dt, nsteps, box=REFERENCE_BOX, threads=0):
        """nsteps steps; returns (pos, vel, rho, prs) in input-index order."""
        pos = _f32(pos, (-1, 3))
        n = len(pos)
        vel = None if vel is None else _f32(vel, (n, 3))
        bx = None if box is None else _f32(box)
        po = np.zeros((n, 3), np.float32)
        vo = np.zeros((n, 3), np.float32)
        ro = np.zeros(n, np.float32)
        pr = np.zeros(n, np.float32)
        rc = self.lib.orc_run(n, pos, _ptr(vel), _f32(args), _ptr(bx), C.c_float(dt),
                              int(nsteps), int(threads), _ptr(po), _ptr(vo), _ptr(ro),
                              _ptr(pr))
        if rc != 0:
            raise RuntimeError("oracle run failed: %d" % rc)
        return po, vo, ro, pr

    def fields_f64(self, pos, vel, args):
        pos = _f32(pos, (-1, 3))
        n = len(pos)
        vel = None if vel is None else _f32(vel, (n, 3))
        rho = np.zeros(n, np.float64)
        prs = np.zeros(n, np.float64)
        force = np.zeros((n, 3), np.float64)
        rc = self.lib.orc_fields_f64(n, pos, _ptr(vel), _f32(args), rho, prs, force)
        if rc != 0:
            raise RuntimeError("oracle f64 failed: %d" % rc)
        return rho, prs, force


# ------------------------------------------------------------------ workloads
#
# numpy restatements of the product's workload generators, so that the CPU
# arms (bench.py --impl reference, the oracle side of the parity tests) can
# build the same inputs without loading the product library.  A test checks
# each against the product's own generator bit for bit.

GAMMA = np.uint64(0x9E3779B97F4A7C15)
SPACING = 0.05
JITTER = 0.0025
DT = 0.002


def mix64(z):
    """SplitMix64's output function over uint64 arrays."""
    z = np.asarray(z, np.uint64)
    with np.errstate(over="ignore"):
        z = z + GAMMA
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def lattice(nx, ny, nz, origin, spacing, jitter, seed):
    """The jittered cubic lattice of sphx_lattice: row idx = (k * ny + j) * nx + i,
    coordinate a = origin[a] + ijk[a] * spacing + (2u - 1) * jitter with u the top
    24 bits of SplitMix64(seed + (3 idx + a + 1) * gamma) times 2^-24, every
    operation in float32 in that order."""
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


def config_args(gas_const=20.0, viscosity=1.0):
    """SPHSettings constructor floats of the benchmark configurations (mass 0.125,
    rest density 1000, k, mu, h 0.1, g -9.8, tension 0) as float32."""
    return np.array([0.125, 1000.0, gas_const, viscosity, 0.1, -9.8, 0.0], np.float32)


def dambreak(nx, ny=None, nz=None, box_scale=(2.5, 1.25, 1.25), seed=0, h=0.1,
             spacing=SPACING, jitter=JITTER):
    """A dam-break block: nx*ny*nz lattice particles in the corner of a box
    box_scale times the block edges (x, z centred on 0, floor y = 0, no
    ceiling, damping 0.5, offset 1e-4), starting one spacing inside the
    reflection planes.  Returns (positions (n, 3) float32, box as the 9-float
    oracle array)."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    f = lambda v: float(np.float32(v))  # the box is stored as float32
    edges = np.array([nx, ny, nz], np.float64) * spacing
    dims = edges * np.array(box_scale)
    box = np.array([f(-dims[0] / 2), f(dims[0] / 2), 0.0, f(dims[1]), f(-dims[2] / 2),
                    f(dims[2] / 2), f(0.5), f(0.0001), 0.0], np.float32)
    origin = (f(float(box[0]) + h + spacing), f(float(box[2]) + h + spacing),
              f(float(box[4]) + h + spacing))
    return lattice(nx, ny, nz, origin, spacing, jitter, seed), box


def build():
    """Builds the oracle libraries (restatement always; reference where present)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("build_oracle", os.path.join(HERE, "build_oracle.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build_port(), mod.build_ref()
