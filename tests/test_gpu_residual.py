"""Residual norms of gcfd_step (the printed residual of euler.go:814-849):
the sums of squares are reduced in FP64 in a fixed order, so the norms are
the same bit for bit when a step is repeated from the same state, and on the
mixed path they are accurate to FP64 level, not FP32 level.

The reference for the RMS is numpy's FP64 norm of the state difference around
one step.  On the FP64 path that difference is the increment up to one
rounding of the state (~1e-16 |Q|); on the mixed path the increment is the FP32
value that was added to the compensated (~48-bit) state, so the difference
reproduces it to ~1e-14 |Q|.  The tolerances (1e-9 relative) sit far above
those and far below what an FP32 accumulation of the squares gives (~1e-7).
"""
import numpy as np
import pytest

from gocfd_gb300 import meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D

pytestmark = pytest.mark.gpu


def _params(N):
    return InputParameters2D(CFL=1.0, FluxType="roe", InitType="ivortex", PolynomialOrder=N, FinalTime=1e9,
                             MaxIterations=10 ** 9)


@pytest.mark.parametrize("precision,N", [("fp64", 3), ("fp32", 4), ("fp32", 2), ("tf32x3", 4)])
def test_residual_rms_is_fp64_accurate_and_deterministic(precision, N):
    mesh = meshes.vortex_box(40, jitter=0.1, seed=3)
    with Euler(_params(N), mesh, 1, precision=precision, vortex_center=(0.0, 0.0)) as gpu:
        gpu.step(3)
        q0 = gpu.get_global_state()
        t0 = gpu.time
        runs = []
        for _ in range(3):
            gpu.set_global_state(q0)
            gpu.time = t0
            info = gpu.step(1)
            runs.append((np.array(info["resid_rms"]), np.array(info["resid_absmax"]), gpu.get_global_state()))
        for rms, ab, q1 in runs[1:]:
            assert np.array_equal(rms.view(np.uint64), runs[0][0].view(np.uint64)), (rms, runs[0][0])
            assert np.array_equal(ab, runs[0][1])
        rms, ab, q1 = runs[0]
        d = (q1 - q0).reshape(4, -1)
        ref_rms = np.sqrt((d * d).sum(axis=1) / d.shape[1])
        ref_ab = np.abs(d).max(axis=1)
        assert np.all(ref_rms > 0)
        assert np.allclose(rms, ref_rms, rtol=1e-9, atol=0), (rms, ref_rms, rms / ref_rms - 1)
        assert np.allclose(ab, ref_ab, rtol=1e-9, atol=0)


def test_residual_rms_deterministic_with_pipelined_stage_kernel():
    mesh = meshes.vortex_box(48, jitter=0.1, seed=5)  # K = 4608, K % 4 == 0
    with Euler(_params(4), mesh, 1, precision="fp32", vortex_center=(0.0, 0.0)) as gpu:
        gpu.set_stage_pipeline(True)
        assert gpu.stage_pipeline()
        gpu.step(2)
        q0 = gpu.get_global_state()
        t0 = gpu.time
        out = []
        for _ in range(2):
            gpu.set_global_state(q0)
            gpu.time = t0
            out.append(np.array(gpu.step(1)["resid_rms"]))
            q1 = gpu.get_global_state()
        assert np.array_equal(out[0].view(np.uint64), out[1].view(np.uint64))
        d = (q1 - q0).reshape(4, -1)
        assert np.allclose(out[0], np.sqrt((d * d).mean(axis=1)), rtol=1e-9, atol=0)
