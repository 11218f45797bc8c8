"""Python binding of the sphx C-ABI (include/sphx.h) over ctypes.

Thin by design: every call goes straight to lib/libsphx.so, which must be
built (``build_sphx.py``); importing this module on a machine without the
library raises, and creating a scene without a usable GPU raises
:class:`SphxError` — there is no CPU path.

Also defines the benchmark / test workloads as data: dam-break lattice blocks
(jittered cubic lattices, SplitMix64-seeded) in boxes whose walls follow the
reference's convention (reflection at bound +- h, floor at y = 0, no ceiling;
src/sph.cpp:139-176).
"""
import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsphx.so")

SPHX_OK = 0
ERRORS = {-1: "INVALID", -2: "CUDA", -3: "NOMEM", -4: "DOMAIN", -5: "OVERFLOW", -6: "STATE"}


class SphxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("sphx error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


class Settings(C.Structure):
    """SPHSettings constructor arguments (SPHSystem.h:15-17)."""
    _fields_ = [(n, C.c_float) for n in
                ("mass", "rest_density", "gas_const", "viscosity", "h", "g", "tension")]


class Derived(C.Structure):
    _fields_ = [(n, C.c_float) for n in
                ("poly6", "spiky_grad", "spiky_lap", "gas_constant", "mass", "h2", "self_dens",
                 "rest_density", "viscosity", "h", "g", "tension", "mass_poly6_product")] + [
                    ("sphere_scale", C.c_float * 16)]


class Box(C.Structure):
    _fields_ = [(n, C.c_float) for n in
                ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax", "damping", "offset")] + [
                    ("has_ceiling", C.c_int)]

    def as_array(self):
        """9-float form (xmin, xmax, ymin, ymax, zmin, zmax, damping, offset, ceiling)."""
        return np.array([self.xmin, self.xmax, self.ymin, self.ymax, self.zmin, self.zmax,
                         self.damping, self.offset, float(self.has_ceiling)], np.float32)


class Options(C.Structure):
    _fields_ = [("reorder_interval", C.c_int), ("use_graph", C.c_int), ("device", C.c_int),
                ("stream", C.c_void_p), ("grid_ymax", C.c_float), ("grid_dims", C.c_int * 3),
                ("grid_origin", C.c_int * 3), ("max_cell_occupancy", C.c_uint32),
                ("density_threads", C.c_int), ("force_threads", C.c_int),
                ("neighbor_slots", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("settings", Settings), ("box", Box), ("n", C.c_size_t),
                ("pos3", C.c_void_p), ("vel3", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("density_threads", C.c_int), ("force_threads", C.c_int),
                ("reorder_interval", C.c_int), ("ms_per_step", C.c_double)]


class LatticeDesc(C.Structure):
    _fields_ = [("nx", C.c_uint32), ("ny", C.c_uint32), ("nz", C.c_uint32),
                ("origin", C.c_float * 3), ("spacing", C.c_float), ("jitter", C.c_float),
                ("seed", C.c_uint64)]


class DeviceView(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("vel", C.c_void_p), ("force", C.c_void_p),
                ("rho_prs", C.c_void_p), ("id", C.c_void_p), ("n", C.c_size_t),
                ("stream", C.c_void_p)]


class KernelTimes(C.Structure):
    _fields_ = [("sort_ms", C.c_double), ("density_ms", C.c_double), ("force_ms", C.c_double),
                ("steps", C.c_uint64), ("launches", C.c_uint64)]


class ServerOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("steps_per_tick", C.c_int),
                ("max_scenes", C.c_int), ("dt", C.c_float), ("device", C.c_int)]


class Request(C.Structure):
    _fields_ = [("settings", Settings), ("box", Box), ("n", C.c_size_t), ("pos3", C.c_void_p),
                ("vel3", C.c_void_p), ("nsteps", C.c_int)]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int), ("steps_done", C.c_int), ("submit_s", C.c_double),
                ("admit_s", C.c_double), ("done_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("ticks", C.c_uint64),
                ("relayouts", C.c_uint64), ("particle_steps", C.c_uint64),
                ("live_scenes", C.c_size_t), ("queued", C.c_size_t),
                ("bytes_in_use", C.c_size_t), ("elapsed_s", C.c_double),
                ("layout_s", C.c_double), ("step_s", C.c_double), ("readout_s", C.c_double)]


_lib = None


def lib():
    """Loads lib/libsphx.so once (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError("libsphx.so not built: %s (run build_sphx.py)" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, P = C.c_void_p, C.POINTER
    sig = {
        "sphx_version": (C.c_char_p, []),
        "sphx_last_error": (C.c_char_p, []),
        "sphx_settings_reference": (None, [P(Settings)]),
        "sphx_box_reference": (None, [P(Box)]),
        "sphx_options_default": (None, [P(Options)]),
        "sphx_derive": (C.c_int, [P(Settings), P(Derived)]),
        "sphx_hash": (C.c_uint32, [C.c_int32, C.c_int32, C.c_int32]),
        "sphx_cell": (None, [C.c_float, C.c_float, C.c_float, C.c_float, vp]),
        "sphx_collision_flags": (C.c_uint32, [C.c_int32, C.c_int32, C.c_int32, C.c_uint32]),
        "sphx_lattice": (C.c_int, [P(LatticeDesc), vp]),
        "sphx_reference_scene": (C.c_int, [C.c_size_t, C.c_float, vp]),
        "sphx_create": (C.c_int, [P(Settings), P(Box), P(Options), C.c_size_t, vp, vp, P(vp)]),
        "sphx_create_batch": (C.c_int, [P(SceneDesc), C.c_size_t, P(Options), P(vp)]),
        "sphx_scene_count": (C.c_size_t, [vp]),
        "sphx_create_lattice": (C.c_int, [P(Settings), P(Box), P(Options), P(LatticeDesc), P(vp)]),
        "sphx_replace_scene": (C.c_int, [vp, C.c_size_t, P(SceneDesc), P(LatticeDesc)]),
        "sphx_set_settings": (C.c_int, [vp, C.c_size_t, P(Settings), P(Box)]),
        "sphx_scene_range": (C.c_int, [vp, C.c_size_t, P(C.c_size_t), P(C.c_size_t)]),
        "sphx_read_scene": (C.c_int, [vp, C.c_size_t, vp, vp, vp, vp, vp]),
        "sphx_get_tuning": (C.c_int, [vp, P(Tuning)]),
        "sphx_set_tuning": (C.c_int, [vp, P(Tuning)]),
        "sphx_autotune": (C.c_int, [vp, C.c_float, C.c_int, C.c_char_p, P(Tuning)]),
        "sphx_density_static": (C.c_int, [P(Settings), vp, C.c_size_t, vp, vp, vp]),
        "sphx_destroy": (C.c_int, [vp]),
        "sphx_count": (C.c_size_t, [vp]),
        "sphx_set_state": (C.c_int, [vp, vp, vp]),
        "sphx_step": (C.c_int, [vp, C.c_float, C.c_int]),
        "sphx_synchronize": (C.c_int, [vp]),
        "sphx_read_state": (C.c_int, [vp, vp, vp, vp, vp, vp]),
        "sphx_read_transforms": (C.c_int, [vp, vp]),
        "sphx_read_cells": (C.c_int, [vp, vp, vp]),
        "sphx_neighbor_digest": (C.c_int, [vp, vp, vp]),
        "sphx_walk_stats": (C.c_int, [vp, vp, vp]),
        "sphx_device_state": (C.c_int, [vp, P(DeviceView)]),
        "sphx_update_particles": (C.c_int, [vp, vp, C.c_size_t, P(Settings), P(Box), C.c_float]),
        "sphx_update_particles_release": (C.c_int, []),
        "sphx_server_options_default": (None, [P(ServerOptions)]),
        "sphx_server_create": (C.c_int, [P(ServerOptions), P(vp)]),
        "sphx_server_submit": (C.c_int, [vp, P(Request), P(C.c_uint64)]),
        "sphx_server_status": (C.c_int, [vp, C.c_uint64, P(RequestStatus)]),
        "sphx_server_wait": (C.c_int, [vp, C.c_uint64, C.c_double]),
        "sphx_server_result": (C.c_int, [vp, C.c_uint64, vp, vp, vp, vp]),
        "sphx_server_stats_get": (C.c_int, [vp, P(ServerStats)]),
        "sphx_server_inject_failure": (C.c_int, [vp, C.c_int]),
        "sphx_server_destroy": (C.c_int, [vp]),
        "sphx_set_profiling": (C.c_int, [vp, C.c_int]),
        "sphx_get_kernel_times": (C.c_int, [vp, P(KernelTimes)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != SPHX_OK:
        raise SphxError(rc, lib().sphx_last_error().decode())
    return rc


def _ptr(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _f32(a, n=None):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a.reshape(-1, 3) if n is None else a.reshape(n, 3)


def settings(mass, rest_density, gas_const, viscosity, h, g, tension=0.0):
    return Settings(mass, rest_density, gas_const, viscosity, h, g, tension)


def reference_settings():
    s = Settings()
    lib().sphx_settings_reference(C.byref(s))
    return s


def reference_box():
    b = Box()
    lib().sphx_box_reference(C.byref(b))
    return b


def default_options(**kw):
    o = Options()
    lib().sphx_options_default(C.byref(o))
    for k, v in kw.items():
        if k in ("grid_dims", "grid_origin"):
            getattr(o, k)[:] = list(v)
        else:
            setattr(o, k, v)
    return o


def derive(s):
    d = Derived()
    _check(lib().sphx_derive(C.byref(s), C.byref(d)))
    return d


def args_array(s):
    """The 7 constructor floats as a float32 array (oracle argument form)."""
    return np.array([s.mass, s.rest_density, s.gas_const, s.viscosity, s.h, s.g, s.tension],
                    np.float32)


def hash18(cx, cy, cz):
    return lib().sphx_hash(int(cx), int(cy), int(cz))


def cell(x, y, z, h):
    out = np.zeros(3, np.int32)
    lib().sphx_cell(x, y, z, h, _ptr(out))
    return out


def lattice(nx, ny, nz, origin, spacing, jitter, seed):
    d = LatticeDesc(nx, ny, nz, (C.c_float * 3)(*origin), spacing, jitter, seed)
    out = np.zeros((nx * ny * nz, 3), np.float32)
    _check(lib().sphx_lattice(C.byref(d), _ptr(out)))
    return out


def reference_scene(width, h):
    out = np.zeros((width ** 3, 3), np.float32)
    _check(lib().sphx_reference_scene(width, h, _ptr(out)))
    return out


# ------------------------------------------------------------------ workloads

SPACING = 0.05
JITTER = 0.0025  # +-5% of the spacing
DT = 0.002


def config_settings(gas_const=20.0, viscosity=1.0):
    """Physics constants shared by every benchmark configuration."""
    return settings(0.125, 1000.0, gas_const, viscosity, 0.1, -9.8, 0.0)


def dambreak(nx, ny=None, nz=None, box_scale=(2.5, 1.25, 1.25), box_dims=None, seed=0,
             h=0.1, spacing=SPACING, jitter=JITTER):
    """A jittered lattice block of nx*ny*nz particles in the corner of a box.

    The box is x, z centred on 0 with the floor at y = 0 (no ceiling); its
    extents are ``box_dims`` or ``box_scale`` times the block edges.  The
    block starts one spacing inside the reflection planes (bound + h).
    Returns (positions (n, 3) float32, Box)."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    edges = np.array([nx, ny, nz], np.float64) * spacing
    dims = np.array(box_dims if box_dims is not None else edges * np.array(box_scale))
    b = Box(-dims[0] / 2, dims[0] / 2, 0.0, dims[1], -dims[2] / 2, dims[2] / 2, 0.5, 0.0001, 0)
    origin = (b.xmin + h + spacing, b.ymin + h + spacing, b.zmin + h + spacing)
    pos = lattice(nx, ny, nz, origin, spacing, jitter, seed)
    return pos, b


# ------------------------------------------------------------------ reference seam

PARTICLE_DTYPE = np.dtype([("position", np.float32, 3), ("velocity", np.float32, 3),
                           ("acceleration", np.float32, 3), ("force", np.float32, 3),
                           ("density", np.float32), ("pressure", np.float32),
                           ("hash", np.uint16), ("_pad", np.uint16)])
assert PARTICLE_DTYPE.itemsize == 60  # Particle.h:4-10


def particles_from(pos, vel=None):
    """An array of the reference's 60-byte Particle records."""
    rec = np.zeros(len(pos), PARTICLE_DTYPE)
    rec["position"] = pos
    if vel is not None:
        rec["velocity"] = vel
    return rec


def update_particles(records, s, dt, box=None, transforms=None):
    """One step in place over Particle records (updateParticlesGPU's contract)."""
    assert records.dtype == PARTICLE_DTYPE and records.flags["C_CONTIGUOUS"]
    _check(lib().sphx_update_particles(C.c_void_p(records.ctypes.data),
                                       _ptr(transforms), len(records), C.byref(s),
                                       C.byref(box) if box is not None else None, dt))


def release_update_particles():
    _check(lib().sphx_update_particles_release())


def batch_scenes(count=512, seed=0, nmin=1000, nmax=65536):
    """The batched workload: `count` dam-break blocks with particle counts
    log-uniform in [nmin, nmax], block aspect ratios uniform in [0.5, 2],
    gas constant uniform in [10, 40] and viscosity uniform in [0.5, 3]
    (other constants as config_settings), each in a box 2.5 / 1.25 / 1.25
    times its block edges.  Returns a list of (Settings, pos, Box)."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        target = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        aspect = rng.uniform(0.5, 2.0, 3)
        c = (target / aspect.prod()) ** (1.0 / 3.0)
        nx, ny, nz = (max(2, int(round(c * a))) for a in aspect)
        s = config_settings(gas_const=float(rng.uniform(10, 40)), viscosity=float(rng.uniform(0.5, 3)))
        pos, box = dambreak(nx, ny, nz, seed=seed * 100003 + k)
        out.append((s, pos, box))
    return out


# ------------------------------------------------------------------ scene handle

class Scene:
    """A resident scene (one sphx_handle)."""

    def __init__(self, s, box, pos, vel=None, options=None):
        pos = _f32(pos)
        n = len(pos)
        vel = None if vel is None else _f32(vel, n)
        self.n = n
        self.settings = s
        self.box = box if box is not None else reference_box()
        self.options = options if options is not None else default_options()
        h = C.c_void_p()
        _check(lib().sphx_create(C.byref(s), C.byref(self.box), C.byref(self.options), n,
                                 _ptr(pos), _ptr(vel), C.byref(h)))
        self.h = h

    @classmethod
    def batch(cls, scenes, options=None):
        """One handle over many scenes: scenes is a list of (Settings, pos, Box)
        or (Settings, pos, Box, vel)."""
        self = cls.__new__(cls)
        self.options = options if options is not None else default_options()
        keep = []
        descs = (SceneDesc * len(scenes))()
        for k, sc in enumerate(scenes):
            s, pos, box = sc[0], _f32(sc[1]), sc[2]
            vel = None if len(sc) < 4 or sc[3] is None else _f32(sc[3], len(pos))
            keep += [pos, vel]
            descs[k] = SceneDesc(s, box, len(pos), pos.ctypes.data,
                                 None if vel is None else vel.ctypes.data)
        h = C.c_void_p()
        _check(lib().sphx_create_batch(descs, len(scenes), C.byref(self.options), C.byref(h)))
        self.h = h
        self.n = int(lib().sphx_count(h))
        self.settings = None
        self.box = None
        return self

    @classmethod
    def from_lattice(cls, s, box, desc, options=None):
        """A scene whose lattice (LatticeDesc) is generated on the device."""
        self = cls.__new__(cls)
        self.options = options if options is not None else default_options()
        h = C.c_void_p()
        _check(lib().sphx_create_lattice(C.byref(s), C.byref(box), C.byref(self.options),
                                         C.byref(desc), C.byref(h)))
        self.h = h
        self.n = int(lib().sphx_count(h))
        self.settings = s
        self.box = box
        return self

    def replace_scene(self, k, s, box, pos=None, vel=None, lattice=None):
        keep = []
        if lattice is None:
            pos = _f32(pos)
            vel = None if vel is None else _f32(vel, len(pos))
            keep = [pos, vel]
            d = SceneDesc(s, box, len(pos), pos.ctypes.data, None if vel is None else vel.ctypes.data)
            _check(lib().sphx_replace_scene(self.h, k, C.byref(d), None))
        else:
            d = SceneDesc(s, box, 0, None, None)
            _check(lib().sphx_replace_scene(self.h, k, C.byref(d), C.byref(lattice)))
        self.n = int(lib().sphx_count(self.h))
        del keep

    def set_settings(self, k, s, box=None):
        _check(lib().sphx_set_settings(self.h, k, C.byref(s),
                                       C.byref(box) if box is not None else None))

    @property
    def scene_count(self):
        return int(lib().sphx_scene_count(self.h))

    def scene_range(self, k):
        first, count = C.c_size_t(), C.c_size_t()
        _check(lib().sphx_scene_range(self.h, k, C.byref(first), C.byref(count)))
        return first.value, count.value

    def read_scene(self, k):
        n = self.scene_range(k)[1]
        out = {"pos": np.zeros((n, 3), np.float32), "vel": np.zeros((n, 3), np.float32),
               "force": np.zeros((n, 3), np.float32), "rho": np.zeros(n, np.float32),
               "prs": np.zeros(n, np.float32)}
        _check(lib().sphx_read_scene(self.h, k, _ptr(out["pos"]), _ptr(out["vel"]),
                                     _ptr(out["rho"]), _ptr(out["prs"]), _ptr(out["force"])))
        return out

    def tuning(self):
        t = Tuning()
        _check(lib().sphx_get_tuning(self.h, C.byref(t)))
        return t

    def set_tuning(self, density_threads=128, force_threads=128, reorder_interval=1):
        t = Tuning(density_threads, force_threads, reorder_interval, 0.0)
        _check(lib().sphx_set_tuning(self.h, C.byref(t)))

    def autotune(self, dt=DT, trial_steps=4, cache_path=None):
        t = Tuning()
        _check(lib().sphx_autotune(self.h, dt, trial_steps,
                                   None if cache_path is None else cache_path.encode(),
                                   C.byref(t)))
        return t

    def close(self):
        if self.h:
            lib().sphx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dt=DT, nsteps=1):
        _check(lib().sphx_step(self.h, dt, nsteps))

    def synchronize(self):
        _check(lib().sphx_synchronize(self.h))

    def set_state(self, pos, vel=None):
        pos = _f32(pos, self.n)
        vel = None if vel is None else _f32(vel, self.n)
        _check(lib().sphx_set_state(self.h, _ptr(pos), _ptr(vel)))

    def read(self):
        """Returns dict of pos, vel, force (n, 3) and rho, prs (n,) in id order."""
        n = self.n
        out = {"pos": np.zeros((n, 3), np.float32), "vel": np.zeros((n, 3), np.float32),
               "force": np.zeros((n, 3), np.float32), "rho": np.zeros(n, np.float32),
               "prs": np.zeros(n, np.float32)}
        _check(lib().sphx_read_state(self.h, _ptr(out["pos"]), _ptr(out["vel"]),
                                     _ptr(out["rho"]), _ptr(out["prs"]), _ptr(out["force"])))
        return out

    def transforms(self):
        out = np.zeros((self.n, 16), np.float32)
        _check(lib().sphx_read_transforms(self.h, _ptr(out)))
        return out

    def cells(self):
        c = np.zeros((self.n, 3), np.int32)
        hsh = np.zeros(self.n, np.uint16)
        _check(lib().sphx_read_cells(self.h, _ptr(c), _ptr(hsh)))
        return c, hsh

    def neighbor_digest(self):
        cnt = np.zeros(self.n, np.uint32)
        dig = np.zeros(self.n, np.uint64)
        _check(lib().sphx_neighbor_digest(self.h, _ptr(cnt), _ptr(dig)))
        return cnt, dig

    def walk_stats(self):
        """(candidates whose r^2 the walk evaluates, accepted neighbour visits)
        for the current positions, summed over all particles."""
        t = C.c_uint64()
        a = C.c_uint64()
        _check(lib().sphx_walk_stats(self.h, C.byref(t), C.byref(a)))
        return t.value, a.value

    def device_view(self):
        v = DeviceView()
        _check(lib().sphx_device_state(self.h, C.byref(v)))
        return v

    def set_profiling(self, on=True):
        _check(lib().sphx_set_profiling(self.h, int(bool(on))))

    def kernel_times(self):
        t = KernelTimes()
        _check(lib().sphx_get_kernel_times(self.h, C.byref(t)))
        return t


class Server:
    """The continuous-batching request loop (sphx_server_*)."""

    REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3

    def __init__(self, budget_bytes=None, steps_per_tick=10, max_scenes=0, dt=DT, device=0):
        o = ServerOptions()
        lib().sphx_server_options_default(C.byref(o))
        if budget_bytes is not None:
            o.hbm_budget_bytes = int(budget_bytes)
        o.steps_per_tick = steps_per_tick
        o.max_scenes = max_scenes
        o.dt = dt
        o.device = device
        h = C.c_void_p()
        _check(lib().sphx_server_create(C.byref(o), C.byref(h)))
        self.h = h
        self.sizes = {}

    def submit(self, s, box, pos, nsteps, vel=None):
        pos = _f32(pos)
        vel = None if vel is None else _f32(vel, len(pos))
        q = Request(s, box, len(pos), pos.ctypes.data, None if vel is None else vel.ctypes.data,
                    int(nsteps))
        t = C.c_uint64()
        _check(lib().sphx_server_submit(self.h, C.byref(q), C.byref(t)))
        self.sizes[t.value] = len(pos)
        return t.value

    def status(self, ticket):
        st = RequestStatus()
        _check(lib().sphx_server_status(self.h, ticket, C.byref(st)))
        return st

    def wait(self, ticket, timeout=120.0):
        _check(lib().sphx_server_wait(self.h, ticket, timeout))

    def result(self, ticket):
        n = self.sizes.pop(ticket)
        out = {"pos": np.zeros((n, 3), np.float32), "vel": np.zeros((n, 3), np.float32),
               "rho": np.zeros(n, np.float32), "prs": np.zeros(n, np.float32)}
        _check(lib().sphx_server_result(self.h, ticket, _ptr(out["pos"]), _ptr(out["vel"]),
                                        _ptr(out["rho"]), _ptr(out["prs"])))
        return out

    def inject_failure(self, code=-2):
        """Makes the worker's next tick fail with `code` (host-side injection)."""
        _check(lib().sphx_server_inject_failure(self.h, code))

    def stats(self):
        st = ServerStats()
        _check(lib().sphx_server_stats_get(self.h, C.byref(st)))
        return st

    def close(self):
        if self.h:
            lib().sphx_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

