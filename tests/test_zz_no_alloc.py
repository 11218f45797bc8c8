"""sphx_density_static — the entry point for callers that cannot allocate
device memory (for example a plugin running inside a frame with a fixed GPU
memory budget): density and pressure of device-resident positions, computed
with scratch kept in a static device array.

It is checked, through the C-ABI, against the resident entry point
(sphx_create + sphx_step + sphx_read_state), whose step computes density and
pressure from the same positions, on two calls in a row so that the second
call runs on whatever the first one left in the shared array.  The file is
named to be collected last."""
import ctypes as C

import numpy as np
import pytest

from _util import REL_TOL, rel_err

pytestmark = pytest.mark.gpu


def resident_density(sphx, s, pos, box):
    with sphx.Scene(s, box, pos) as sc:
        sc.step(sphx.DT, 1)
        out = sc.read()
    return out["rho"], out["prs"]


def static_density(sphx, s, pos):
    import torch
    L = sphx.lib()
    L.sphx_density_static.restype = C.c_int
    L.sphx_density_static.argtypes = [C.POINTER(sphx.Settings), C.c_void_p, C.c_size_t,
                                      C.c_void_p, C.c_void_p, C.c_void_p]
    n = len(pos)
    p4 = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    p4[:, :3] = torch.from_numpy(pos).cuda()
    rho = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    prs = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    rc = L.sphx_density_static(C.byref(s), p4.data_ptr(), n, rho.data_ptr(), prs.data_ptr(),
                               C.c_void_p(stream.cuda_stream))
    assert rc == 0, L.sphx_last_error().decode()
    return rho.cpu().numpy(), prs.cpu().numpy()


def test_static_scratch_entry_point_matches_resident_path(sphx_lib):
    sphx = sphx_lib
    s = sphx.config_settings()
    scenes = [sphx.dambreak(30, box_dims=(3.0, 2.0, 2.0), seed=1),   # 27,000 particles
              sphx.dambreak(24, box_dims=(2.0, 2.0, 2.0), seed=2)]   # 13,824: fewer than call 1
    for pos, box in scenes:
        rho_s, prs_s = static_density(sphx, s, pos)
        rho_r, prs_r = resident_density(sphx, s, pos, box)
        assert np.isfinite(rho_s).all() and np.isfinite(prs_s).all()
        assert rel_err(rho_s, rho_r) < REL_TOL
        assert rel_err(prs_s, prs_r) < REL_TOL


def test_static_scratch_aliased_grid_matches_resident_path(sphx_lib):
    """A block 7 m long in x at h = 0.1 covers cells -35..34, wider than the
    entry point's fixed 64-cell grid: cells then share grid slots and the walk
    takes its slower, non-monotone path.  Results must not change."""
    sphx = sphx_lib
    s = sphx.config_settings()
    pos, box = sphx.dambreak(140, 6, 6, box_dims=(7.6, 2.0, 2.0), seed=3)
    assert pos[:, 0].max() - pos[:, 0].min() > 6.4
    rho_s, prs_s = static_density(sphx, s, pos)
    rho_r, prs_r = resident_density(sphx, s, pos, box)
    assert rel_err(rho_s, rho_r) < REL_TOL
    assert rel_err(prs_s, prs_r) < REL_TOL


def test_static_scratch_rejects_non_finite_position(sphx_lib):
    import torch
    sphx = sphx_lib
    L = sphx.lib()
    s = sphx.config_settings()
    pos, _ = sphx.dambreak(10, seed=4)
    p4 = torch.zeros((len(pos), 4), dtype=torch.float32, device="cuda")
    p4[:, :3] = torch.from_numpy(pos).cuda()
    p4[17, 1] = float("nan")
    out = torch.zeros(len(pos), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    rc = L.sphx_density_static(C.byref(s), p4.data_ptr(), len(pos), out.data_ptr(), out.data_ptr(),
                               None)
    assert rc == -4  # SPHX_ERR_DOMAIN
    # the array is usable again by the next call
    rho_s, _ = static_density(sphx, s, pos)
    assert np.isfinite(rho_s).all()


def test_static_scratch_rejects_oversize(sphx_lib):
    import torch
    sphx = sphx_lib
    L = sphx.lib()
    s = sphx.config_settings()
    n = (1 << 17) + 1
    buf = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    out = torch.zeros(n, dtype=torch.float32, device="cuda")
    rc = L.sphx_density_static(C.byref(s), buf.data_ptr(), n, out.data_ptr(), out.data_ptr(), None)
    assert rc == -1
    assert b"131072" in L.sphx_last_error()
