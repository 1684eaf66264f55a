"""sam_gpu_vel_max_noalloc: the vel_max entry point for callers that cannot
call cudaMalloc (their device memory belongs to another allocator, or their
step loop must not stall on an allocation).  Here torch's allocator plays that
caller's role: it owns the input field and the output, and the library call
itself allocates nothing.  The results must match the existing vel_max entry
point (sam_gpu_vel_max, which stages the host field through its own device
buffers) on two calls in a row, the second on a different field, so the
shared scratch array carries nothing from one call to the next.

This file is collected last so that, if it fails, a run stopping at the first
failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from sam_gb300 import SamGpu
from sam_gb300.sam_gpu import load_library

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the tolerance of the FP64 parity tests for full runs


def _noalloc(lib, torch, u_host, lu, stream):
    nx, ny, nz = u_host.shape[:3]
    # device copies owned by torch's allocator; Fortran order -> transpose view
    u_dev = torch.from_numpy(np.ascontiguousarray(u_host.transpose(3, 2, 1, 0))).cuda()
    out = torch.full((16,), -1.0, dtype=torch.float64, device="cuda")
    rc = lib.sam_gpu_vel_max_noalloc(C.c_void_p(u_dev.data_ptr()), nx, ny, nz, lu, C.c_void_p(out.data_ptr()),
                                     C.c_void_p(stream))
    assert rc == 0, lib.sam_gpu_error_string()
    torch.cuda.current_stream().synchronize()
    return out.cpu().numpy()


def test_vel_max_noalloc_matches_vel_max(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = load_library()
    nx, ny, nz, lu = 48, 40, 36, 4
    g = SamGpu(nx=nx, ny=ny, nz=nz, i_strat=1, buoy_fac_z=1.0, lapse=1.0)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(2024)
    for call in range(2):
        u = np.asfortranarray(rng.standard_normal((nx, ny, nz, lu)) * (1.0 + call) + 0.1 * call)
        ref = g.vel_max(u)
        got = _noalloc(lib, torch, u, lu, stream)
        np.testing.assert_allclose(got[0:4], ref["u_avg"], rtol=TOL, atol=TOL * np.abs(u).max())
        np.testing.assert_allclose(got[4:8], ref["u_var"], rtol=TOL)
        np.testing.assert_array_equal(got[8:12], ref["u_max"])
        assert abs(got[12] - ref["energy"]) <= TOL * ref["energy"]
        assert got[13] == 0.0
    g.close()


def test_vel_max_noalloc_rejects_oversize(gpu_lib):
    lib = load_library()
    dummy = C.c_void_p(1)  # never dereferenced: the size check comes first
    rc = lib.sam_gpu_vel_max_noalloc(dummy, 8, 8, 4097, 4, dummy, None)
    assert rc == -1
    assert b"SAM_GPU_NOALLOC_MAX_PLANES" in lib.sam_gpu_error_string()
