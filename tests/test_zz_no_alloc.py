"""gcfd_residual_norms_static (the entry point that allocates nothing) against
the residual norms gcfd_step reports for the same increments, two calls in a
row so that the second call runs on the scratch array the first one left.

The increments given to it are the difference of two device snapshots of the
FP64 state around one step; they equal the step's own increments to within
one rounding of the state (~1e-16 |Q|), far inside the FP64 tolerance used
here (1e-10 relative to the largest |R| of the variable).
"""
import ctypes as C

import numpy as np
import pytest

from gocfd_gb300 import _lib, meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D

pytestmark = pytest.mark.gpu

RTOL = 1e-10


def static_norms(lib, dR, Np, K, stream):
    mx, ab, rms = (C.c_double * 4)(), (C.c_double * 4)(), (C.c_double * 4)()
    rc = lib.gcfd_residual_norms_static(C.c_void_p(dR.data_ptr()), Np, K, C.c_void_p(stream), mx, ab, rms)
    assert rc == 0, (rc, lib.gcfd_last_error(None))
    return np.array(mx[:]), np.array(ab[:]), np.array(rms[:])


def test_static_norms_match_step_norms_twice():
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    mesh = meshes.vortex_box(12, jitter=0.1)
    ip = InputParameters2D(CFL=1.0, FluxType="roe", InitType="ivortex", PolynomialOrder=3, FinalTime=1e9,
                           Minf=0.1, Gamma=1.4, MaxIterations=10 ** 9)
    with Euler(ip, mesh, 1, precision="fp64", vortex_center=(0.0, 0.0)) as gpu:
        lib = gpu.lib
        Np, K = gpu.Np, gpu.K
        before = torch.empty((4, Np, K), dtype=torch.float64, device="cuda")
        after = torch.empty_like(before)
        stream = torch.cuda.current_stream().cuda_stream
        for call in range(2):
            assert lib.gcfd_get_state_device(gpu.ctx, C.c_void_p(before.data_ptr())) == 0
            info = gpu.step(1)
            assert lib.gcfd_get_state_device(gpu.ctx, C.c_void_p(after.data_ptr())) == 0
            torch.cuda.synchronize()  # the snapshot copies run on the solver's stream
            dR = (after - before).contiguous()
            mx, ab, rms = static_norms(lib, dR, Np, K, stream)
            ref_mx = np.array(info["resid_max"])
            ref_ab = np.array(info["resid_absmax"])
            ref_rms = np.array(info["resid_rms"])
            scale = np.maximum(ref_ab, 1e-300)
            assert np.all(np.abs(mx - ref_mx) <= RTOL * scale), (call, mx, ref_mx)
            assert np.all(np.abs(ab - ref_ab) <= RTOL * scale), (call, ab, ref_ab)
            assert np.all(np.abs(rms - ref_rms) <= RTOL * scale), (call, rms, ref_rms)
            assert np.all(ab > 0.0)


@pytest.mark.parametrize("Np,K", [(16, 40000), (16, 33554432 // 16 - 3)])
def test_static_norms_of_random_increments(Np, K):
    """Sizes with more than 256 first-pass blocks (the second pass loops) and
    just under the fixed limit, against torch's own FP64 reductions; after one
    warm-up call (module loading), repeated calls leave the device's free
    memory unchanged, i.e. they allocate nothing."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    dR = torch.randn((4, Np, K), dtype=torch.float64, device="cuda", generator=gen)
    dR[1] *= 1e-3
    dR[3] += 0.5
    stream = torch.cuda.current_stream().cuda_stream
    static_norms(lib, dR, Np, K, stream)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    outs = [static_norms(lib, dR, Np, K, stream) for _ in range(3)]
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    flat = dR.reshape(4, -1)
    ref_mx = flat.amax(dim=1).cpu().numpy()
    ref_ab = flat.abs().amax(dim=1).cpu().numpy()
    ref_rms = torch.sqrt((flat * flat).sum(dim=1) / flat.shape[1]).cpu().numpy()
    for mx, ab, rms in outs:
        assert np.array_equal(mx, ref_mx)
        assert np.array_equal(ab, ref_ab)
        assert np.allclose(rms, ref_rms, rtol=1e-12, atol=0), (rms, ref_rms)
        assert np.array_equal(rms, outs[0][2])  # fixed reduction order: same bits every call


def test_static_norms_reject_sizes_beyond_the_limit():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    limit = 33554432  # GCFD_RESID_STATIC_MAX_POINTS
    mx = (C.c_double * 4)()
    rc = lib.gcfd_residual_norms_static(C.c_void_p(buf.data_ptr()), 16, limit // 16 + 1, None, mx, None, None)
    assert rc == -2  # GCFD_ERR_SHAPE, rejected on the host before any launch
    assert b"GCFD_RESID_STATIC_MAX_POINTS" in lib.gcfd_last_error(None)
